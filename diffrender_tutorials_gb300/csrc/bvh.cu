// Scene flattening and the hierarchy over the flattened triangles.
//
// prepare_scene() is the device counterpart of Scene::prepare_for_render
// (common_src/scene_utils.cpp:98-173): it applies each instance transform to
// its mesh, transforms normals by the inverse transpose, and then writes the
// triangles the caster tests.  Those are transformed once more by their
// instance transform, as BruteForce3D::GetNearestHit does
// (raytrace_src/raytrace3d_bf.cpp:116-125); for identity transforms this is
// exact.  Each triangle is stored as (A, B-A, C-A): the same differences the
// caster forms, so the intersection arithmetic is unchanged.
//
// build_bvh() builds the topology of a binary hierarchy, one triangle per
// leaf, with one of three builders: a binned SAH on the host over every
// triangle; the two-level build for instanced scenes (one SAH per mesh,
// shared by its instances, under one over the instances, the shape of the
// reference's Embree scene, raytrace_src/raytrace3d_embree.cpp:35-50); or a
// linear BVH on the device (Karras 2012: Morton codes of triangle centroids,
// LSD radix sort, binary radix tree).  refit_bvh() recomputes every box
// bottom-up and runs after each parameter update, since vertex positions
// move but the triangles do not; the rebuild_bvh_* functions renew the
// topology from moved vertices, overlapped with later work.  Boxes are
// padded so that the traversal never culls a triangle the brute-force test
// would accept.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>
#include <future>

#include "engine.h"

namespace drgb {

// Per block: its transform and the inverse transpose used for normals.
__device__ __forceinline__ void block_tr_body(const BlockDev* blocks, int b, const float* const* mesh_tr,
                                              float* block_tr) {
  const BlockDev bd = blocks[b];
  const float* tr = mesh_tr[bd.mesh] + 16 * bd.inst;
  float inv[16];
  mat_inverse44(tr, inv);
  float* o = block_tr + 32 * b;
  for (int i = 0; i < 16; i++) o[i] = tr[i];
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) o[16 + 4 * c + r] = inv[4 * r + c];  // transpose
}

__global__ void k_block_tr(const BlockDev* blocks, int n_blocks, const float* const* mesh_tr, float* block_tr) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_blocks) return;
  block_tr_body(blocks, b, mesh_tr, block_tr);
}

// Flattened vertex arrays (prepare_for_render's per-instance loop).
__device__ __forceinline__ void flatten_body(int g, const int* vblock, const BlockDev* blocks, const MeshSrc* src,
                                             const float* block_tr, float4* pos, float4* orig, float4* col,
                                             float4* nrm, float2* tc, float4* tan) {
  const int b = vblock[g];
  const BlockDev bd = blocks[b];
  const int k = g - bd.vert_off;
  const MeshSrc s = src[bd.mesh];
  const float* tr = block_tr + 32 * b;
  const f3 v = mk(s.v[3 * k], s.v[3 * k + 1], s.v[3 * k + 2]);
  const f3 p = mat_pt(tr, v);
  pos[g] = make_float4(p.x, p.y, p.z, 0.0f);
  orig[g] = make_float4(v.x, v.y, v.z, 0.0f);
  col[g] = s.col ? make_float4(s.col[3 * k], s.col[3 * k + 1], s.col[3 * k + 2], 0.0f) : make_float4(0, 0, 0, 0);
  if (s.nrm) {
    const f3 nn = mat_pt(tr + 16, mk(s.nrm[3 * k], s.nrm[3 * k + 1], s.nrm[3 * k + 2]));
    nrm[g] = make_float4(nn.x, nn.y, nn.z, 0.0f);
  } else {
    nrm[g] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  }
  tc[g] = s.tc ? make_float2(s.tc[2 * k], s.tc[2 * k + 1]) : make_float2(0.0f, 0.0f);
  if (tan) {  // tangents by the inverse transpose, default (0,1,0) (scene_utils.cpp:133,167-168)
    const f3 tt = s.tan ? mat_pt(tr + 16, mk(s.tan[3 * k], s.tan[3 * k + 1], s.tan[3 * k + 2])) : mk(0.0f, 1.0f, 0.0f);
    tan[g] = make_float4(tt.x, tt.y, tt.z, 0.0f);
  }
}

__global__ void k_flatten(const int* vblock, int n, const BlockDev* blocks, const MeshSrc* src, const float* block_tr,
                          float4* pos, float4* orig, float4* col, float4* nrm, float2* tc, float4* tan) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  flatten_body(g, vblock, blocks, src, block_tr, pos, orig, col, nrm, tc, tan);
}

// ---------------------------------------------------------------------------
// LBVH topology.
// ---------------------------------------------------------------------------
__device__ __forceinline__ f3 traced_vertex(const float4* pos, const float* block_tr, int b, int g) {
  return mat_pt(block_tr + 32 * b, ld3(pos, g));
}

__global__ void k_centroid_bounds(const int4* tri_v, int n, const float4* pos, const float* block_tr, float* bounds) {
  __shared__ float smin[3][256], smax[3][256];
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int4 tv = tri_v[t];
    const f3 a = traced_vertex(pos, block_tr, tv.w, tv.x);
    const f3 b = traced_vertex(pos, block_tr, tv.w, tv.y);
    const f3 c = traced_vertex(pos, block_tr, tv.w, tv.z);
    const float cx = (a.x + b.x + c.x) * (1.0f / 3.0f), cy = (a.y + b.y + c.y) * (1.0f / 3.0f),
                cz = (a.z + b.z + c.z) * (1.0f / 3.0f);
    lo[0] = fminf(lo[0], cx); lo[1] = fminf(lo[1], cy); lo[2] = fminf(lo[2], cz);
    hi[0] = fmaxf(hi[0], cx); hi[1] = fmaxf(hi[1], cy); hi[2] = fmaxf(hi[2], cz);
  }
  for (int a = 0; a < 3; a++) { smin[a][threadIdx.x] = lo[a]; smax[a][threadIdx.x] = hi[a]; }
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int a = 0; a < 3; a++) {
        smin[a][threadIdx.x] = fminf(smin[a][threadIdx.x], smin[a][threadIdx.x + s]);
        smax[a][threadIdx.x] = fmaxf(smax[a][threadIdx.x], smax[a][threadIdx.x + s]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int a = 0; a < 3; a++) { bounds[a] = smin[a][0]; bounds[3 + a] = smax[a][0]; }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void k_morton(const int4* tri_v, int n, const float4* pos, const float* block_tr, const float* bounds,
                         uint32_t* keys, int* vals) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int4 tv = tri_v[t];
  const f3 a = traced_vertex(pos, block_tr, tv.w, tv.x);
  const f3 b = traced_vertex(pos, block_tr, tv.w, tv.y);
  const f3 c = traced_vertex(pos, block_tr, tv.w, tv.z);
  float q[3] = {(a.x + b.x + c.x) * (1.0f / 3.0f), (a.y + b.y + c.y) * (1.0f / 3.0f), (a.z + b.z + c.z) * (1.0f / 3.0f)};
  uint32_t code = 0;
  for (int k = 0; k < 3; k++) {
    const float ext = bounds[3 + k] - bounds[k];
    float f = ext > 0.0f ? (q[k] - bounds[k]) / ext : 0.5f;
    f = fminf(fmaxf(f, 0.0f), 1.0f);
    const uint32_t xi = min((uint32_t)(f * 1024.0f), 1023u);
    code |= expand_bits(xi) << (2 - k);
  }
  keys[t] = code;
  vals[t] = t;
}

// LSD radix sort of (key, value) pairs, 8-bit digits, stable.
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint32_t* keys, int n, int shift, uint32_t* hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
  for (int i = threadIdx.x; i < RS_TILE; i += RS_THREADS)
    if (base + i < n) atomicAdd(&h[(keys[base + i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive prefix sum of hist[0, m) in place (one block): tiles of 16,384
// counters, 16 consecutive ones per thread (four 16-byte loads, so a warp
// reads 2 KB contiguously), a warp-shuffle scan of the thread sums, and a
// carry from tile to tile.  hist must be 16-byte aligned (a buffer start).
// Exclusive scan of the tile hist[base, base + 16384) in place (1024 threads,
// 16 counters each), offset by `carry`; returns the tile's total.
__device__ __forceinline__ uint32_t scan_tile(uint32_t* hist, int m, int base, uint32_t carry, uint32_t* wsum) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int i0 = base + tid * 16;
  uint32_t v[16];
  if (i0 + 16 <= m) {
    const uint4* p = reinterpret_cast<const uint4*>(hist + i0);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint4 x = p[q];
      v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = i0 + k < m ? hist[i0 + k] : 0u;
  }
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < 16; k++) {
    const uint32_t x = v[k];
    v[k] = sum;
    sum += x;
  }
  uint32_t inc = sum;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = wsum[lane];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    wsum[lane] = w;
  }
  __syncthreads();
  const uint32_t before = carry + (warp ? wsum[warp - 1] : 0u) + (inc - sum);
  if (i0 + 16 <= m) {
    uint4* p = reinterpret_cast<uint4*>(hist + i0);
#pragma unroll
    for (int q = 0; q < 4; q++)
      p[q] = make_uint4(v[4 * q] + before, v[4 * q + 1] + before, v[4 * q + 2] + before, v[4 * q + 3] + before);
  } else {
#pragma unroll
    for (int k = 0; k < 16; k++)
      if (i0 + k < m) hist[i0 + k] = v[k] + before;
  }
  const uint32_t total = wsum[31];
  __syncthreads();  // wsum is rewritten by the next tile
  return total;
}

constexpr int RS_SCAN_TILE = 1024 * 16;

__global__ void __launch_bounds__(1024) k_rs_scan(uint32_t* hist, int m) {
  __shared__ uint32_t wsum[32];
  uint32_t carry = 0;
  for (int base = 0; base < m; base += RS_SCAN_TILE) carry += scan_tile(hist, m, base, carry, wsum);
}

// Several tiles: one block scans each tile on its own and keeps its total in
// the slot past the counters; a second pass adds the totals of the tiles
// before it to every counter of a tile.
__global__ void __launch_bounds__(1024) k_rs_scan_tiles(uint32_t* hist, int m, uint32_t* totals) {
  __shared__ uint32_t wsum[32];
  const uint32_t t = scan_tile(hist, m, blockIdx.x * RS_SCAN_TILE, 0u, wsum);
  if (threadIdx.x == 0) totals[blockIdx.x] = t;
}

__global__ void __launch_bounds__(1024) k_rs_scan_offsets(uint32_t* hist, int m, const uint32_t* totals) {
  __shared__ uint32_t off;
  if (threadIdx.x == 0) {
    uint32_t o = 0;
    for (int b = 0; b < (int)blockIdx.x; b++) o += totals[b];
    off = o;
  }
  __syncthreads();
  if (blockIdx.x == 0) return;
  const int i0 = blockIdx.x * RS_SCAN_TILE + threadIdx.x * 16;
  if (i0 + 16 <= m) {
    uint4* p = reinterpret_cast<uint4*>(hist + i0);
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint4 x = p[q];
      p[q] = make_uint4(x.x + off, x.y + off, x.z + off, x.w + off);
    }
  } else {
    for (int k = 0; k < 16; k++)
      if (i0 + k < m) hist[i0 + k] += off;
  }
}

// `hist` has room for scan_scratch(m) counters: m, then one total per tile.
void launch_rs_scan(uint32_t* hist, int m, cudaStream_t s) {
  const int tiles = (m + RS_SCAN_TILE - 1) / RS_SCAN_TILE;
  if (tiles <= 1) {
    k_rs_scan<<<1, 1024, 0, s>>>(hist, m);
    count_launch();
    return;
  }
  uint32_t* totals = hist + ((m + 3) & ~3);
  k_rs_scan_tiles<<<tiles, 1024, 0, s>>>(hist, m, totals);
  k_rs_scan_offsets<<<tiles, 1024, 0, s>>>(hist, m, totals);
  count_launch(2);
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint32_t* kin, const int* vin, uint32_t* kout,
                                                           int* vout, int n, int shift, const uint32_t* hist) {
  __shared__ uint32_t offs[256];
  __shared__ uint32_t wcnt[RS_THREADS / 32][257];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  offs[tid] = hist[tid * gridDim.x + blockIdx.x];
  const int base = blockIdx.x * RS_TILE;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < RS_ITEMS; r++) {
    for (int i = tid; i < (RS_THREADS / 32) * 257; i += RS_THREADS) (&wcnt[0][0])[i] = 0u;
    __syncthreads();
    const int idx = base + r * RS_THREADS + tid;
    const bool valid = idx < n;
    const uint32_t key = valid ? kin[idx] : 0u;
    const int val = valid ? vin[idx] : 0;
    const uint32_t digit = valid ? ((key >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const uint32_t rank = __popc(peers & lt);
    if ((__ffs(peers) - 1) == lane) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t off = offs[digit] + rank;
      for (int w = 0; w < warp; w++) off += wcnt[w][digit];
      kout[off] = key;
      vout[off] = val;
    }
    __syncthreads();
    uint32_t tot = 0;
    for (int w = 0; w < RS_THREADS / 32; w++) tot += wcnt[w][tid];
    offs[tid] += tot;
    __syncthreads();
  }
}

__device__ __forceinline__ int lbvh_delta(const uint32_t* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const unsigned long long a = ((unsigned long long)keys[i] << 32) | (unsigned)i;
  const unsigned long long b = ((unsigned long long)keys[j] << 32) | (unsigned)j;
  return __clzll(a ^ b);
}

// Binary radix tree (Karras 2012, Algorithm 4): internal node i, leaves ~k.
__global__ void k_karras(const uint32_t* keys, int n, float4* nodes, int* leaf_parent, int* node_parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (lbvh_delta(keys, n, i, i + 1) - lbvh_delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = lbvh_delta(keys, n, i, i - d);
  int lmax = 2;
  while (lbvh_delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (lbvh_delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = lbvh_delta(keys, n, i, j);
  int s = 0;
  for (int div = 2;; div <<= 1) {
    const int t = (l + div - 1) / div;
    if (lbvh_delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
  }
  const int gamma = i + s * d + min(d, 0);
  const int left = (min(i, j) == gamma) ? ~gamma : gamma;
  const int right = (max(i, j) == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  nodes[4 * i + 3] = make_float4(__int_as_float(left), __int_as_float(right), 0.0f, 0.0f);
  if (left < 0) leaf_parent[~left] = i; else node_parent[left] = i;
  if (right < 0) leaf_parent[~right] = i; else node_parent[right] = i;
  if (i == 0) node_parent[0] = -1;
}

// ---------------------------------------------------------------------------
// Leaf triangles + bottom-up refit.
// ---------------------------------------------------------------------------
struct Box {
  float lx, hx, ly, hy, lz, hz;
};

__device__ __forceinline__ void write_child(float4* nodes, int parent, int slot, const Box& b) {
  float* n = reinterpret_cast<float*>(nodes + 4 * parent);
  if (slot == 0) {
    n[0] = b.lx; n[1] = b.hx; n[2] = b.ly; n[3] = b.hy; n[8] = b.lz; n[9] = b.hz;
  } else {
    n[4] = b.lx; n[5] = b.hx; n[6] = b.ly; n[7] = b.hy; n[10] = b.lz; n[11] = b.hz;
  }
}

// Leaf k: its triangle's traced vertices (A, e1, e2) and, in leaf_of, the
// leaf slot of that triangle (refreshed with every refit, so it follows any
// topology change); then the boxes up the tree.
__device__ __forceinline__ void leaf_refit_body(int k, const int* perm, int n, const int4* tri_v, const float4* pos,
                                                const float* block_tr, float4* tri, float4* nodes,
                                                const int* leaf_parent, const int* node_parent, int* counters,
                                                int* leaf_of) {
  const int t = perm[k];
  leaf_of[t] = k;
  const int4 tv = tri_v[t];
  const f3 A = traced_vertex(pos, block_tr, tv.w, tv.x);
  const f3 B = traced_vertex(pos, block_tr, tv.w, tv.y);
  const f3 C = traced_vertex(pos, block_tr, tv.w, tv.z);
  const f3 e1 = B - A, e2 = C - A;
  tri[3 * k + 0] = make_float4(A.x, A.y, A.z, __int_as_float(t));
  tri[3 * k + 1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
  tri[3 * k + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
  if (n == 1) return;
  Box b;
  b.lx = fminf(A.x, fminf(B.x, C.x)); b.hx = fmaxf(A.x, fmaxf(B.x, C.x));
  b.ly = fminf(A.y, fminf(B.y, C.y)); b.hy = fmaxf(A.y, fmaxf(B.y, C.y));
  b.lz = fminf(A.z, fminf(B.z, C.z)); b.hz = fmaxf(A.z, fmaxf(B.z, C.z));
  const float ext = fmaxf(b.hx - b.lx, fmaxf(b.hy - b.ly, b.hz - b.lz));
  const float mag = fmaxf(fmaxf(fmaxf(fabsf(b.lx), fabsf(b.hx)), fmaxf(fabsf(b.ly), fabsf(b.hy))),
                          fmaxf(fabsf(b.lz), fabsf(b.hz)));
  const float pad = ext * 1e-5f + mag * 2e-6f + 1e-20f;
  b.lx -= pad; b.ly -= pad; b.lz -= pad; b.hx += pad; b.hy += pad; b.hz += pad;
  int child = ~k;
  int p = leaf_parent[k];
  while (p >= 0) {
    const float4 c = __ldcg(nodes + 4 * p + 3);
    const int slot = (__float_as_int(c.x) == child) ? 0 : 1;
    write_child(nodes, p, slot, b);
    __threadfence();
    if (atomicAdd(counters + p, 1) == 0) return;  // the sibling finishes this node
    __threadfence();
    const float4 n0 = __ldcg(nodes + 4 * p + 0), n1 = __ldcg(nodes + 4 * p + 1), n2 = __ldcg(nodes + 4 * p + 2);
    b.lx = fminf(n0.x, n1.x); b.hx = fmaxf(n0.y, n1.y);
    b.ly = fminf(n0.z, n1.z); b.hy = fmaxf(n0.w, n1.w);
    b.lz = fminf(n2.x, n2.z); b.hz = fmaxf(n2.y, n2.w);
    child = p;
    p = node_parent[p];
  }
}

// `light`, `tiles_state` (may be null): the light-space cells and the
// raster pass's tile lists no longer hold the geometry.
__global__ void k_leaves_refit(const int* perm, int n, const int4* tri_v, const float4* pos, const float* block_tr,
                               float4* tri, float4* nodes, const int* leaf_parent, const int* node_parent,
                               int* counters, int* leaf_of, LightGrid* light, uint32_t* tiles_state) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0 && light) light->valid = 0;
  if (k == 0 && tiles_state) *tiles_state &= ~2u;
  if (k >= n) return;
  leaf_refit_body(k, perm, n, tri_v, pos, block_tr, tri, nodes, leaf_parent, node_parent, counters, leaf_of);
}

// 4-wide node of binary internal node p (layout in JobDev::nodes4; used by
// builds with -DDRGB_BVH4): slots
// 0-1 hold child 0's two children when child 0 is internal, else child 0
// itself and an unused slot; slots 2-3 the same for child 1.  The boxes are
// copied from the refitted binary nodes, so they stay conservative.
__device__ __forceinline__ void collapse4_body(const float4* nodes, int p, float4* nodes4) {
  float lx[4], hx[4], ly[4], hy[4], lz[4], hz[4];
  int link[4];
  const float4 q0 = __ldcg(nodes + 4 * p + 0), q1 = __ldcg(nodes + 4 * p + 1);
  const float4 q2 = __ldcg(nodes + 4 * p + 2), q3 = __ldcg(nodes + 4 * p + 3);
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int c = __float_as_int(side ? q3.y : q3.x);
    const int s0 = 2 * side, s1 = 2 * side + 1;
    if (c >= 0) {
      const float4 a0 = __ldcg(nodes + 4 * c + 0), a1 = __ldcg(nodes + 4 * c + 1);
      const float4 a2 = __ldcg(nodes + 4 * c + 2), a3 = __ldcg(nodes + 4 * c + 3);
      lx[s0] = a0.x; hx[s0] = a0.y; ly[s0] = a0.z; hy[s0] = a0.w; lz[s0] = a2.x; hz[s0] = a2.y;
      link[s0] = __float_as_int(a3.x);
      lx[s1] = a1.x; hx[s1] = a1.y; ly[s1] = a1.z; hy[s1] = a1.w; lz[s1] = a2.z; hz[s1] = a2.w;
      link[s1] = __float_as_int(a3.y);
    } else {
      const float4 b = side ? q1 : q0;
      lx[s0] = b.x; hx[s0] = b.y; ly[s0] = b.z; hy[s0] = b.w;
      lz[s0] = side ? q2.z : q2.x;
      hz[s0] = side ? q2.w : q2.y;
      link[s0] = c;
      lx[s1] = hx[s1] = ly[s1] = hy[s1] = lz[s1] = hz[s1] = 0.0f;
      link[s1] = kEmpty4;
    }
  }
  float4* o = nodes4 + 8 * p;
  o[0] = make_float4(lx[0], lx[1], lx[2], lx[3]);
  o[1] = make_float4(hx[0], hx[1], hx[2], hx[3]);
  o[2] = make_float4(ly[0], ly[1], ly[2], ly[3]);
  o[3] = make_float4(hy[0], hy[1], hy[2], hy[3]);
  o[4] = make_float4(lz[0], lz[1], lz[2], lz[3]);
  o[5] = make_float4(hz[0], hz[1], hz[2], hz[3]);
  o[6] = make_float4(__int_as_float(link[0]), __int_as_float(link[1]), __int_as_float(link[2]),
                     __int_as_float(link[3]));
  o[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_collapse4(const float4* nodes, int n_internal, float4* nodes4) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n_internal) collapse4_body(nodes, p, nodes4);
}

// ---- batched forms: one launch over the scenes of many jobs --------------
// The segment tables give, per job, the number of blocks / vertices /
// internal nodes / triangles (Seg::count) and the first chunk of 256.
__global__ void k_b_block_tr(const JobAux* aux, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int b = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (b >= sg.count) return;
  const JobAux& A = aux[sg.job];
  block_tr_body(A.blocks, b, A.tr_tab, A.block_tr);
}

__global__ void k_b_flatten(const JobAux* aux, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int g = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (g >= sg.count) return;
  const JobAux& A = aux[sg.job];
  flatten_body(g, A.vblock, A.blocks, A.src, A.block_tr, A.pos, A.orig, A.col, A.nrm, A.tc, A.tan);
}

__global__ void k_b_zero_counters(const JobAux* aux, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int i = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (i >= sg.count) return;
  aux[sg.job].counters[i] = 0;
}

__global__ void k_b_refit(const JobAux* aux, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int k = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (k >= sg.count) return;
  const JobAux& A = aux[sg.job];
  leaf_refit_body(k, A.perm, A.n_tris, A.tri_v, A.pos, A.block_tr, A.tri, A.nodes, A.leaf_parent, A.node_parent,
                  A.counters, A.leaf_of);
}

// segment table over the jobs' internal node counts
__global__ void k_b_collapse4(const JobAux* aux, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int p = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (p >= sg.count) return;
  const JobAux& A = aux[sg.job];
  collapse4_body(A.nodes, p, A.nodes4);
}

// Flatten + refit of every job of a batch (segment tables built by the host:
// blocks, vertices, internal nodes and triangles per job).
void launch_b_prepare(const JobAux* d_aux, const Seg* segs[4], const int nsegs[4], const int chunks[4],
                      cudaStream_t s) {
  if (chunks[0] > 0) k_b_block_tr<<<chunks[0], 256, 0, s>>>(d_aux, segs[0], nsegs[0]);
  if (chunks[1] > 0) k_b_flatten<<<chunks[1], 256, 0, s>>>(d_aux, segs[1], nsegs[1]);
  if (chunks[2] > 0) k_b_zero_counters<<<chunks[2], 256, 0, s>>>(d_aux, segs[2], nsegs[2]);
  if (chunks[3] > 0) k_b_refit<<<chunks[3], 256, 0, s>>>(d_aux, segs[3], nsegs[3]);
#ifdef DRGB_BVH4
  if (chunks[2] > 0) k_b_collapse4<<<chunks[2], 256, 0, s>>>(d_aux, segs[2], nsegs[2]);
  count_launch();
#endif
  count_launch(4);
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
void flatten_scene(Job& J, cudaStream_t s) {
  if (J.n_vertices == 0) return;
  k_block_tr<<<(J.n_blocks + 63) / 64, 64, 0, s>>>(J.blocks.p, J.n_blocks, J.tr_tab.p, J.block_tr.p);
  k_flatten<<<(J.n_vertices + 255) / 256, 256, 0, s>>>(J.vblock.p, J.n_vertices, J.blocks.p, J.src_tab.p,
                                                      J.block_tr.p, J.pos.p, J.orig.p, J.col.p, J.nrm.p, J.tc.p,
                                                      J.tan.p);
  count_launch(2);
}

void prepare_scene(Job& J, cudaStream_t s) {
  flatten_scene(J, s);
  refit_bvh(J, s);
}

void commit_scene(Job& J, cudaStream_t s) {
  flatten_scene(J, s);
  build_bvh(J, s);
  refit_bvh(J, s);
}

// A new topology from the flattened positions of the last prepare_scene (the
// optimiser's current vertices); same sizes, so every device pointer and a
// captured iteration graph stay valid.
void rebuild_bvh(Job& J, cudaStream_t s) {
  J.topo_builder = -1;  // defeats the same-triangles cache
  build_bvh(J, s);
  refit_bvh(J, s);
}

static void host_topology(int builder, const float4* pos, const float* block_tr, const std::vector<int4>& tri_v,
                          const std::vector<BlockDev>& blocks, int n_vertices, int n, std::vector<float4>& links,
                          std::vector<int>& perm, std::vector<int>& leaf_parent, std::vector<int>& node_parent);

// The pieces of an overlapped rebuild: the current vertices copied out
// behind the enqueued work, the topology built on a host thread into pinned
// buffers, and copied in (and refitted) in stream order.
static void topo_copy_out(Job& J, TopoRebuild& T, cudaStream_t s) {
  if (!T.ev) DRGB_CUDA(cudaEventCreateWithFlags(&T.ev, cudaEventDisableTiming));
  T.pos.reserve((size_t)J.n_vertices);
  DRGB_CUDA(cudaMemcpyAsync(T.pos.p, J.pos.p, sizeof(float4) * J.n_vertices, cudaMemcpyDeviceToHost, s));
  T.block_tr.reserve(32 * (size_t)J.n_blocks);
  DRGB_CUDA(cudaMemcpyAsync(T.block_tr.p, J.block_tr.p, sizeof(float) * 32 * J.n_blocks, cudaMemcpyDeviceToHost, s));
  T.builder = J.bvh_builder;
  DRGB_CUDA(cudaEventRecord(T.ev, s));
  const int n = J.n_tris;
  T.nodes.reserve(4 * (size_t)(n - 1));
  T.perm.reserve(n);
  T.leaf_parent.reserve(n);
  T.node_parent.reserve(n - 1);
}

// wait_copy: the thread first waits for the copy-out (its device is `dev`).
static void topo_start_build(Job& J, TopoRebuild& T, bool wait_copy) {
  TopoRebuild* t = &T;
  const std::vector<int4>* tri_v = &J.h_tri_v;
  const std::vector<BlockDev>* blocks = &J.h_blocks;
  const int nv = J.n_vertices, n = J.n_tris;
  int dev = 0;
  DRGB_CUDA(cudaGetDevice(&dev));
  T.task = std::async(std::launch::async, [t, tri_v, blocks, nv, n, wait_copy, dev] {
    if (wait_copy) {
      DRGB_CUDA(cudaSetDevice(dev));
      DRGB_CUDA(cudaEventSynchronize(t->ev));
    }
    std::vector<float4> links;
    std::vector<int> perm, leaf_parent, node_parent;
    host_topology(t->builder, t->pos.p, t->block_tr.p, *tri_v, *blocks, nv, n, links, perm, leaf_parent,
                  node_parent);
    std::fill(t->nodes.p, t->nodes.p + 4 * (size_t)(n - 1), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int i = 0; i < n - 1; i++) t->nodes.p[4 * (size_t)i + 3] = links[i];
    std::memcpy(t->perm.p, perm.data(), sizeof(int) * n);
    std::memcpy(t->leaf_parent.p, leaf_parent.data(), sizeof(int) * n);
    std::memcpy(t->node_parent.p, node_parent.data(), sizeof(int) * (n - 1));
  });
}

static void topo_copy_in(Job& J, TopoRebuild& T, cudaStream_t s) {
  T.task.get();
  const int n = J.n_tris;
  DRGB_CUDA(cudaMemcpyAsync(J.nodes.p, T.nodes.p, sizeof(float4) * 4 * (n - 1), cudaMemcpyHostToDevice, s));
  DRGB_CUDA(cudaMemcpyAsync(J.perm.p, T.perm.p, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  DRGB_CUDA(cudaMemcpyAsync(J.leaf_parent.p, T.leaf_parent.p, sizeof(int) * n, cudaMemcpyHostToDevice, s));
  DRGB_CUDA(cudaMemcpyAsync(J.node_parent.p, T.node_parent.p, sizeof(int) * (n - 1), cudaMemcpyHostToDevice, s));
  refit_bvh(J, s);
  J.topo_tri_v = J.h_tri_v;
  J.topo_builder = T.builder;
  T.stage = 0;
}

void rebuild_bvh_begin(Job& J, cudaStream_t s) {
  const int n = J.n_tris;
  if (J.bvh_builder == 0 || n <= 1) {  // a device build blocks nothing
    rebuild_bvh(J, s);
    return;
  }
  if (!J.topo_async) J.topo_async.reset(new TopoRebuild());
  TopoRebuild& T = *J.topo_async;
  if (T.stage != 0) return;  // the previous one is still on its way
  topo_copy_out(J, T, s);
  T.stage = 1;
}

void rebuild_bvh_poll(Job& J, cudaStream_t s) {
  if (!J.topo_async) return;
  TopoRebuild& T = *J.topo_async;
  if (T.stage == 1) {
    const cudaError_t q = cudaEventQuery(T.ev);
    if (q == cudaErrorNotReady) return;
    DRGB_CUDA(q);
    topo_start_build(J, T, false);
    T.stage = 2;
    return;
  }
  if (T.stage == 2 && T.task.wait_for(std::chrono::seconds(0)) == std::future_status::ready) topo_copy_in(J, T, s);
}

// The optimiser's rebuild, overlapped but deterministic: started after one
// iteration (the vertices of that iteration) and applied after a fixed later
// one, waiting there if the host build has not finished, so that the
// topology each iteration uses does not depend on timing.
void rebuild_bvh_start(Job& J, cudaStream_t s) {
  const int n = J.n_tris;
  if (J.bvh_builder == 0 || n <= 1) {  // a device build blocks nothing
    rebuild_bvh(J, s);
    return;
  }
  if (!J.topo_async) J.topo_async.reset(new TopoRebuild());
  TopoRebuild& T = *J.topo_async;
  if (T.stage == 3) topo_copy_in(J, T, s);  // the previous one first
  rebuild_bvh_discard(J);
  topo_copy_out(J, T, s);
  topo_start_build(J, T, true);
  T.stage = 3;
}

void rebuild_bvh_apply(Job& J, cudaStream_t s) {
  if (J.topo_async && J.topo_async->stage == 3) topo_copy_in(J, *J.topo_async, s);
}

void rebuild_bvh_discard(Job& J) {
  if (!J.topo_async) return;
  TopoRebuild& T = *J.topo_async;
  if (T.task.valid()) {
    try {
      T.task.get();
    } catch (...) {  // the build is dropped, its error with it
    }
  }
  if (T.stage == 1 && T.ev) cudaEventSynchronize(T.ev);  // the copy-out still writes the pinned buffers
  T.stage = 0;
}

void refit_bvh(Job& J, cudaStream_t s) {
  const int n = J.n_tris;
  if (n == 0) return;
  if (n > 1) DRGB_CUDA(cudaMemsetAsync(J.counters.p, 0, sizeof(int) * (n - 1), s));
  k_leaves_refit<<<(n + 127) / 128, 128, 0, s>>>(J.perm.p, n, J.tri_v.p, J.pos.p, J.block_tr.p, J.tri.p, J.nodes.p,
                                                 J.leaf_parent.p, J.node_parent.p, J.counters.p, J.leaf_of.p,
                                                 J.sh_grid.p, J.ra_state.p);
  count_launch();
#ifdef DRGB_BVH4
  if (n > 1) {
    k_collapse4<<<(n - 1 + 127) / 128, 128, 0, s>>>(J.nodes.p, n - 1, J.nodes4.p);
    count_launch();
  }
#endif
}

// Binned SAH build of a hierarchy's topology on the host (16 bins per axis
// over the item centroids, one item per leaf); the boxes are filled by the
// device refit, exactly as for the LBVH.  Outputs the child links of every
// internal node (root 0; a leaf child is ~slot), the leaf permutation (slot
// -> item) and the parent arrays.  Leaf slots and internal nodes are numbered
// in the order the build reaches them.
struct SahItem {
  float lo[3], hi[3], c[3];
};

static void sah_tree(const std::vector<SahItem>& items, std::vector<float4>& links, std::vector<int>& perm,
                     std::vector<int>& leaf_parent, std::vector<int>& node_parent) {
  const int n = (int)items.size();
  if (n < 2) {
    links.assign(1, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    perm.assign((size_t)n, 0);
    leaf_parent.assign((size_t)n, -1);
    node_parent.assign(1, -1);
    return;
  }
  std::vector<int> idx((size_t)n);
  for (int t = 0; t < n; t++) idx[t] = t;
  links.assign((size_t)std::max(n - 1, 1), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
  perm.assign((size_t)n, 0);
  leaf_parent.assign((size_t)n, -1);
  node_parent.assign((size_t)std::max(n - 1, 1), -1);
  constexpr int NB = 16;
  struct Task {
    int b, e, node;
  };
  std::vector<Task> stack{{0, n, 0}};
  int next_node = 1, next_leaf = 0;
  auto area = [](const float* lo, const float* hi) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx * dy + dy * dz + dz * dx;
  };
  while (!stack.empty()) {
    const Task t = stack.back();
    stack.pop_back();
    float cmin[3] = {1e30f, 1e30f, 1e30f}, cmax[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = t.b; i < t.e; i++)
      for (int k = 0; k < 3; k++) {
        cmin[k] = std::min(cmin[k], items[idx[i]].c[k]);
        cmax[k] = std::max(cmax[k], items[idx[i]].c[k]);
      }
    int best_axis = -1, best_split = 0;
    float best_cost = 1e38f;
    for (int ax = 0; ax < 3; ax++) {
      const float ext = cmax[ax] - cmin[ax];
      if (!(ext > 0.0f)) continue;
      int cnt[NB] = {0};
      float blo[NB][3], bhi[NB][3];
      for (int q = 0; q < NB; q++)
        for (int k = 0; k < 3; k++) {
          blo[q][k] = 1e30f;
          bhi[q][k] = -1e30f;
        }
      for (int i = t.b; i < t.e; i++) {
        const SahItem& it = items[idx[i]];
        const int q = std::min(NB - 1, (int)((it.c[ax] - cmin[ax]) / ext * NB));
        cnt[q]++;
        for (int k = 0; k < 3; k++) {
          blo[q][k] = std::min(blo[q][k], it.lo[k]);
          bhi[q][k] = std::max(bhi[q][k], it.hi[k]);
        }
      }
      float rlo[NB][3], rhi[NB][3];
      int rcnt[NB];
      float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
      int c = 0;
      for (int q = NB - 1; q >= 0; q--) {
        c += cnt[q];
        for (int k = 0; k < 3; k++) {
          lo[k] = std::min(lo[k], blo[q][k]);
          hi[k] = std::max(hi[k], bhi[q][k]);
          rlo[q][k] = lo[k];
          rhi[q][k] = hi[k];
        }
        rcnt[q] = c;
      }
      for (int k = 0; k < 3; k++) {
        lo[k] = 1e30f;
        hi[k] = -1e30f;
      }
      c = 0;
      for (int q = 0; q < NB - 1; q++) {
        c += cnt[q];
        for (int k = 0; k < 3; k++) {
          lo[k] = std::min(lo[k], blo[q][k]);
          hi[k] = std::max(hi[k], bhi[q][k]);
        }
        if (c == 0 || rcnt[q + 1] == 0) continue;
        const float cost = c * area(lo, hi) + rcnt[q + 1] * area(rlo[q + 1], rhi[q + 1]);
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = ax;
          best_split = q;
        }
      }
    }
    int mid = (t.b + t.e) / 2;
    if (best_axis >= 0) {
      const float ext = cmax[best_axis] - cmin[best_axis];
      auto it = std::partition(idx.begin() + t.b, idx.begin() + t.e, [&](int tri) {
        return std::min(NB - 1, (int)((items[tri].c[best_axis] - cmin[best_axis]) / ext * NB)) <= best_split;
      });
      mid = (int)(it - idx.begin());
      if (mid == t.b || mid == t.e) mid = (t.b + t.e) / 2;
    }
    int child[2];
    const int rb[2] = {t.b, mid}, re[2] = {mid, t.e};
    for (int side = 0; side < 2; side++) {
      if (re[side] - rb[side] == 1) {
        const int slot = next_leaf++;
        perm[slot] = idx[rb[side]];
        leaf_parent[slot] = t.node;
        child[side] = ~slot;
      } else {
        const int id = next_node++;
        node_parent[id] = t.node;
        child[side] = id;
        stack.push_back(Task{rb[side], re[side], id});
      }
    }
    float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    std::memcpy(&l.x, &child[0], sizeof(int));
    std::memcpy(&l.y, &child[1], sizeof(int));
    links[t.node] = l;
  }
}

// A flattened vertex as traced: after its block's transform (host copy of
// traced_vertex; the build needs no exact value).
static void traced_host(const float4* pos, const float* block_tr, int b, int g, float w[3]) {
  const float4 p = pos[g];
  const float* m = block_tr + 32 * (size_t)b;
  w[0] = p.x * m[0] + p.y * m[4] + p.z * m[8] + m[12];
  w[1] = p.x * m[1] + p.y * m[5] + p.z * m[9] + m[13];
  w[2] = p.x * m[2] + p.y * m[6] + p.z * m[10] + m[14];
}

// Items of n triangles: boxes of their vertices as traced.
static void tri_items(const float4* pos, const float* block_tr, const int4* tri_v, int n, std::vector<SahItem>& items) {
  items.resize((size_t)n);
  for (int t = 0; t < n; t++) {
    const int4 tv = tri_v[t];
    float xa[3], xb[3], xc[3];
    traced_host(pos, block_tr, tv.w, tv.x, xa);
    traced_host(pos, block_tr, tv.w, tv.y, xb);
    traced_host(pos, block_tr, tv.w, tv.z, xc);
    SahItem& it = items[t];
    for (int k = 0; k < 3; k++) {
      it.lo[k] = std::min(xa[k], std::min(xb[k], xc[k]));
      it.hi[k] = std::max(xa[k], std::max(xb[k], xc[k]));
      it.c[k] = 0.5f * (it.lo[k] + it.hi[k]);
    }
  }
}

static void renumber_top(int n, std::vector<float4>& links, std::vector<int>& leaf_parent,
                         std::vector<int>& node_parent);

// One SAH hierarchy over every triangle of the scene.
static void sah_topology(const float4* pos, const float* block_tr, const std::vector<int4>& tri_v, int n,
                         std::vector<float4>& links, std::vector<int>& perm, std::vector<int>& leaf_parent,
                         std::vector<int>& node_parent) {
  std::vector<SahItem> items;
  tri_items(pos, block_tr, tri_v.data(), n, items);
  sah_tree(items, links, perm, leaf_parent, node_parent);
  renumber_top(n, links, leaf_parent, node_parent);
}

// The top levels of the hierarchy take node ids 0..K-1 in breadth-first
// order (the range kernels stage in shared memory); every other node keeps
// its depth-first order after them, so that a subtree stays contiguous.
static void renumber_top(int n, std::vector<float4>& links, std::vector<int>& leaf_parent,
                         std::vector<int>& node_parent) {
#ifdef DRGB_NO_RENUMBER
  return;
#endif
  if (n < 2) return;
  const int K = std::min(n - 1, kTopNodes);
  std::vector<int> order;
  order.reserve((size_t)(n - 1));
  order.push_back(0);
  for (size_t i = 0; i < order.size() && (int)order.size() < K; i++) {
    int c[2];
    std::memcpy(&c[0], &links[order[i]].x, sizeof(int));
    std::memcpy(&c[1], &links[order[i]].y, sizeof(int));
    for (int side = 0; side < 2 && (int)order.size() < K; side++)
      if (c[side] >= 0) order.push_back(c[side]);
  }
  std::vector<char> top((size_t)(n - 1), 0);
  for (int v : order) top[v] = 1;
  for (int v = 0; v < n - 1; v++)
    if (!top[v]) order.push_back(v);
  std::vector<int> new_id((size_t)(n - 1));
  for (int i = 0; i < n - 1; i++) new_id[order[i]] = i;
  std::vector<float4> nl((size_t)(n - 1));
  std::vector<int> np((size_t)(n - 1));
  for (int old = 0; old < n - 1; old++) {
    int c[2];
    std::memcpy(&c[0], &links[old].x, sizeof(int));
    std::memcpy(&c[1], &links[old].y, sizeof(int));
    for (int side = 0; side < 2; side++)
      if (c[side] >= 0) c[side] = new_id[c[side]];
    float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    std::memcpy(&l.x, &c[0], sizeof(int));
    std::memcpy(&l.y, &c[1], sizeof(int));
    nl[new_id[old]] = l;
    np[new_id[old]] = node_parent[old] >= 0 ? new_id[node_parent[old]] : -1;
  }
  links.swap(nl);
  node_parent.swap(np);
  for (int k = 0; k < n; k++) leaf_parent[k] = new_id[leaf_parent[k]];
}


// Two-level build for instanced scenes: one SAH hierarchy per mesh over its
// first instance's triangles, shared by every instance of the mesh, and an
// SAH hierarchy over the instances (their boxes as traced, after the block
// transform); each leaf of the top hierarchy is replaced by a copy of its
// mesh's hierarchy with the instance's triangle and node offsets.  The
// result is one binary hierarchy over world-space boxes and triangles with
// the layout of the flat build (n - 1 internal nodes), so that the traversal
// and its hit arithmetic do not change: only the build is per mesh, and the
// top levels follow the instances.  Cost: one SAH build per mesh plus one
// over the instances, against one over every instance's triangles.
static void two_level_topology(const float4* pos, const float* block_tr, const std::vector<int4>& tri_v,
                               const std::vector<BlockDev>& blocks, int n_vertices, int n,
                               std::vector<float4>& links, std::vector<int>& perm, std::vector<int>& leaf_parent,
                               std::vector<int>& node_parent) {
  const int nb = (int)blocks.size();
  auto tri_end = [&](int b) { return b + 1 < nb ? blocks[b + 1].tri_off : n; };
  auto vert_end = [&](int b) { return b + 1 < nb ? blocks[b + 1].vert_off : n_vertices; };
  // per-mesh hierarchies over local triangle ids (the mesh's index order)
  struct Bottom {
    std::vector<float4> links;
    std::vector<int> perm, leaf_parent, node_parent;
    bool built = false;
  };
  int n_meshes = 0;
  for (const BlockDev& bd : blocks) n_meshes = std::max(n_meshes, bd.mesh + 1);
  std::vector<Bottom> bottom((size_t)n_meshes);
  std::vector<int> inst;  // blocks with triangles: the top hierarchy's items
  std::vector<SahItem> items;
  for (int b = 0; b < nb; b++) {
    const int t0 = blocks[b].tri_off, nt = tri_end(b) - t0;
    if (nt <= 0) continue;
    inst.push_back(b);
    Bottom& B = bottom[blocks[b].mesh];
    if (B.built) continue;
    tri_items(pos, block_tr, tri_v.data() + t0, nt, items);
    sah_tree(items, B.links, B.perm, B.leaf_parent, B.node_parent);
    B.built = true;
  }
  // the instances, boxed as traced
  std::vector<SahItem> top(inst.size());
  for (size_t i = 0; i < inst.size(); i++) {
    const int b = inst[i];
    SahItem& it = top[i];
    for (int k = 0; k < 3; k++) {
      it.lo[k] = 1e30f;
      it.hi[k] = -1e30f;
    }
    for (int g = blocks[b].vert_off; g < vert_end(b); g++) {
      float w[3];
      traced_host(pos, block_tr, b, g, w);
      for (int k = 0; k < 3; k++) {
        it.lo[k] = std::min(it.lo[k], w[k]);
        it.hi[k] = std::max(it.hi[k], w[k]);
      }
    }
    for (int k = 0; k < 3; k++) it.c[k] = 0.5f * (it.lo[k] + it.hi[k]);
  }
  std::vector<float4> tl;
  std::vector<int> tperm, tleaf_parent, tnode_parent;
  sah_tree(top, tl, tperm, tleaf_parent, tnode_parent);
  const int ni = (int)inst.size();
  links.assign((size_t)std::max(n - 1, 1), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
  perm.assign((size_t)n, 0);
  leaf_parent.assign((size_t)n, -1);
  node_parent.assign((size_t)std::max(n - 1, 1), -1);
  auto get = [](const float4& l, int side) {
    int c;
    std::memcpy(&c, side ? &l.y : &l.x, sizeof(int));
    return c;
  };
  auto set = [](float4& l, int side, int c) { std::memcpy(side ? &l.y : &l.x, &c, sizeof(int)); };
  for (int i = 0; i < ni - 1; i++) {
    links[i] = tl[i];
    node_parent[i] = tnode_parent[i];
  }
  int next_node = std::max(ni - 1, 0), next_leaf = 0;
  for (int slot = 0; slot < ni; slot++) {  // the top hierarchy's leaves, in build order
    const int b = inst[tperm[slot]];
    const Bottom& B = bottom[blocks[b].mesh];
    const int t0 = blocks[b].tri_off, nt = tri_end(b) - t0;
    const int node0 = next_node, leaf0 = next_leaf;
    for (int i = 0; i < nt - 1; i++) {
      float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      for (int side = 0; side < 2; side++) {
        const int c = get(B.links[i], side);
        set(l, side, c >= 0 ? c + node0 : ~(~c + leaf0));
      }
      links[node0 + i] = l;
      node_parent[node0 + i] = B.node_parent[i] >= 0 ? B.node_parent[i] + node0 : -1;
    }
    for (int k = 0; k < nt; k++) {
      perm[leaf0 + k] = t0 + B.perm[k];
      leaf_parent[leaf0 + k] = nt > 1 ? B.leaf_parent[k] + node0 : -1;
    }
    next_node += nt - 1;
    next_leaf += nt;
    // hang the instance's root where the top hierarchy had its leaf
    const int root = nt > 1 ? node0 : ~leaf0;
    const int p = ni > 1 ? tleaf_parent[slot] : -1;
    if (p >= 0) {
      set(links[p], get(tl[p], 0) == ~slot ? 0 : 1, root);  // the side in the unmodified top hierarchy
      if (nt > 1) node_parent[node0] = p;
      else leaf_parent[leaf0] = p;
    }
  }
  renumber_top(n, links, leaf_parent, node_parent);
}

// The host builders: 2 the two-level build, 3 one SAH hierarchy over every
// triangle, 1 the two-level build when a mesh has several instances (one
// instance per mesh: a single mesh gives the same hierarchy either way, and
// meshes that overlap in space are better split by triangles).
static void host_topology(int builder, const float4* pos, const float* block_tr, const std::vector<int4>& tri_v,
                          const std::vector<BlockDev>& blocks, int n_vertices, int n, std::vector<float4>& links,
                          std::vector<int>& perm, std::vector<int>& leaf_parent, std::vector<int>& node_parent) {
  bool instanced = false;
  for (const BlockDev& bd : blocks) instanced |= bd.inst > 0;
  if (builder == 2 || (builder == 1 && instanced))
    two_level_topology(pos, block_tr, tri_v, blocks, n_vertices, n, links, perm, leaf_parent, node_parent);
  else
    sah_topology(pos, block_tr, tri_v, n, links, perm, leaf_parent, node_parent);
}

static void build_topology(Job& J, cudaStream_t s);

void build_bvh(Job& J, cudaStream_t s) {
  const int n = J.n_tris;
  // same triangles, same builder: keep the topology, the refit renews the boxes
  const bool same_tris = J.topo_tri_v.size() == J.h_tri_v.size() &&
                         (J.h_tri_v.empty() || std::memcmp(J.topo_tri_v.data(), J.h_tri_v.data(),
                                                           sizeof(int4) * J.h_tri_v.size()) == 0);
  if (J.topo_builder == J.bvh_builder && same_tris && J.nodes.p && J.perm.p) return;
  build_topology(J, s);
}

static void build_topology(Job& J, cudaStream_t s) {
  const int n = J.n_tris;
  J.topo_builder = -1;
  J.tri.alloc(3 * (size_t)std::max(n, 1));
  J.perm.alloc(std::max(n, 1));
  J.leaf_of.alloc(std::max(n, 1));
  J.leaf_parent.alloc(std::max(n, 1));
  J.nodes.alloc(4 * (size_t)std::max(n - 1, 1));
#ifdef DRGB_BVH4
  J.nodes4.alloc(8 * (size_t)std::max(n - 1, 1));
#endif
  J.node_parent.alloc(std::max(n - 1, 1));
  J.counters.alloc(std::max(n - 1, 1));
  if (n == 0) {
    J.root = INT_MIN;
    return;
  }
  if (n == 1) {
    J.root = ~0;
    const int zero = 0, minus1 = -1;
    DRGB_CUDA(cudaMemcpyAsync(J.perm.p, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
    DRGB_CUDA(cudaMemcpyAsync(J.leaf_parent.p, &minus1, sizeof(int), cudaMemcpyHostToDevice, s));
    DRGB_CUDA(cudaStreamSynchronize(s));
    return;
  }
  J.root = 0;
  if (J.bvh_builder != 0) {
    std::vector<float4> pos((size_t)J.n_vertices);
    std::vector<float> block_tr(32 * (size_t)J.n_blocks);
    DRGB_CUDA(cudaMemcpyAsync(pos.data(), J.pos.p, sizeof(float4) * pos.size(), cudaMemcpyDeviceToHost, s));
    DRGB_CUDA(cudaMemcpyAsync(block_tr.data(), J.block_tr.p, sizeof(float) * block_tr.size(), cudaMemcpyDeviceToHost,
                              s));
    DRGB_CUDA(cudaStreamSynchronize(s));
    std::vector<float4> links;
    std::vector<int> perm, leaf_parent, node_parent;
    host_topology(J.bvh_builder, pos.data(), block_tr.data(), J.h_tri_v, J.h_blocks, J.n_vertices, n, links, perm,
                  leaf_parent, node_parent);
    std::vector<float4> nodes(4 * (size_t)(n - 1), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (int i = 0; i < n - 1; i++) nodes[4 * (size_t)i + 3] = links[i];
    DRGB_CUDA(cudaMemcpyAsync(J.nodes.p, nodes.data(), sizeof(float4) * nodes.size(), cudaMemcpyHostToDevice, s));
    DRGB_CUDA(cudaMemcpyAsync(J.perm.p, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    DRGB_CUDA(cudaMemcpyAsync(J.leaf_parent.p, leaf_parent.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    DRGB_CUDA(cudaMemcpyAsync(J.node_parent.p, node_parent.data(), sizeof(int) * (n - 1), cudaMemcpyHostToDevice, s));
    DRGB_CUDA(cudaStreamSynchronize(s));
    J.topo_tri_v = J.h_tri_v;
    J.topo_builder = J.bvh_builder;
    return;
  }
  for (int b = 0; b < 2; b++) {
    J.sort_keys[b].alloc(n);
    J.sort_vals[b].alloc(n);
  }
  const int tiles = (n + RS_TILE - 1) / RS_TILE;
  J.sort_hist.alloc(256 * (size_t)tiles);
  J.bounds.alloc(6);
  k_centroid_bounds<<<1, 256, 0, s>>>(J.tri_v.p, n, J.pos.p, J.block_tr.p, J.bounds.p);
  k_morton<<<(n + 255) / 256, 256, 0, s>>>(J.tri_v.p, n, J.pos.p, J.block_tr.p, J.bounds.p, J.sort_keys[0].p,
                                           J.sort_vals[0].p);
  count_launch(2);
  int cur = 0;
  for (int shift = 0; shift < 32; shift += 8) {
    k_rs_hist<<<tiles, RS_THREADS, 0, s>>>(J.sort_keys[cur].p, n, shift, J.sort_hist.p);
    k_rs_scan<<<1, 1024, 0, s>>>(J.sort_hist.p, 256 * tiles);
    k_rs_scatter<<<tiles, RS_THREADS, 0, s>>>(J.sort_keys[cur].p, J.sort_vals[cur].p, J.sort_keys[cur ^ 1].p,
                                             J.sort_vals[cur ^ 1].p, n, shift, J.sort_hist.p);
    count_launch(3);
    cur ^= 1;
  }
  DRGB_CUDA(cudaMemcpyAsync(J.perm.p, J.sort_vals[cur].p, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  DRGB_CUDA(cudaMemsetAsync(J.nodes.p, 0, sizeof(float4) * 4 * (n - 1), s));
  k_karras<<<(n - 1 + 255) / 256, 256, 0, s>>>(J.sort_keys[cur].p, n, J.nodes.p, J.leaf_parent.p, J.node_parent.p);
  count_launch();
  J.topo_tri_v = J.h_tri_v;
  J.topo_builder = 0;
}

}  // namespace drgb
