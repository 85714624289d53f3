// Edge-sampling boundary term (DiffRender::edge_derivatives,
// src/drender.h:235-425; build_edge_sampler / sample / edge_grad,
// src/drender.cpp:5-87; VS_X_grad / VS_Y_grad, src/functions.cpp:21-163).
//
//   project : VertexShader of every flattened vertex, per view
//   pmf     : edge weights = 3-D length of the projected endpoints
//   cdf     : the sampler's CDF, summed sequentially in edge order so that it
//             is bit-identical to the reference's (one block per view: the
//             block stages chunks in shared memory, one thread runs the chain)
//   select  : replayed random numbers -> edge (upper_bound) -> point ->
//             off-image / small-adjoint rejection; survivors are appended to
//             a queue with one atomic per warp (ballot compaction)
//   shade   : two-sided shading at p -/+ 1e-3 n, (f_in - f_out).dL/dI, chain
//             rule to the world vertices and the instance matrix, scattered
//             with atomics (transform terms summed across the warp first)
//
// Every pass exists in a single-job form (grid over views of one job) and a
// batched form (segment table over the (job, view) pairs of many jobs); both
// run the same per-element code.  Queue entries carry their job index.
#include "engine.h"

namespace drgb {

__device__ __forceinline__ void edge_project_body(const JobDev& J, int view, int v) {
  const CamDev& c = J.cams[view];
  const float4 p = __ldg(J.pos + v);
  float ox, oy;
  vertex_shader(c, p.x, p.y, p.z, ox, oy);
  J.proj[(int64_t)view * J.n_vertices + v] = make_float4(ox, oy, p.z, 0.0f);
}

// Whether a flattened triangle faces the eye (its winding's normal points
// towards it).
__device__ __forceinline__ bool faces_eye(const JobDev& J, int tri, f3 eye) {
  const int4 tv = __ldg(J.tri_v + tri);
  const f3 a = ld3(J.pos, tv.x);
  return dot(cross(ld3(J.pos, tv.y) - a, ld3(J.pos, tv.z) - a), a - eye) < 0.0f;
}

// Sampling weight of an edge: the 3-D length of its projected endpoints
// (build_edge_sampler, drender.cpp:5-22).  Silhouette mode (no reference
// counterpart; the reference samples every edge, drender.h:274-285): an
// edge whose two triangles both face the eye, or both face away, gets
// weight 0 and is never drawn; silhouette and boundary edges keep theirs.
__device__ __forceinline__ void edge_pmf_body(const JobDev& J, int view, int e) {
  const int4 ed = __ldg(J.edges + e);
  const float4* P = J.proj + (int64_t)view * J.n_vertices;
  const float4 a = P[ed.x], b = P[ed.y];
  float w = length(mk(b.x - a.x, b.y - a.y, b.z - a.z));
  if (J.edge_sil) {
    const int2 tt = __ldg(J.edge_tris + e);
    if (tt.y >= 0) {
      const float* m = J.cams[view].wv_inv;
      const f3 eye = mk(m[12], m[13], m[14]);  // the camera position in world space
      if (faces_eye(J, tt.x, eye) == faces_eye(J, tt.y, eye)) w = 0.0f;
    }
  }
  J.pmf[(int64_t)view * J.n_edges + e] = w;
}

// One block (CDF_THREADS): cdf[k+1] = pmf[k] + cdf[k] in edge order, then
// both divided by the total (drender.cpp:5-22).  The running sum is one
// dependent chain of float additions -- the reference's rounding sequence,
// which the sampler's upper_bound must see bit for bit -- so one thread runs
// it, chunk by chunk in shared memory.  Three chunk buffers keep the memory
// traffic off the chain: while thread 0 sums chunk c, warps 1-7 write chunk
// c-1 out and stage chunk c+1.
constexpr int CDF_THREADS = 256;
// 1,024 floats per chunk (12 KB for the three buffers): small enough that a
// CDF block finds room on an SM beside the persistent pixel kernel (with
// 2,048 it did not, and the side-stream CDF ran after the pixel pass).
#ifndef DRGB_CDF_CHUNK
#define DRGB_CDF_CHUNK 1024
#endif
constexpr int CDF_CHUNK = DRGB_CDF_CHUNK;
constexpr int CDF_SMEM = 3 * CDF_CHUNK;  // floats of 16-byte aligned shared memory the caller provides
__device__ __forceinline__ void edge_cdf_body(const JobDev& J, int view, float* sbuf) {
  const int tid = threadIdx.x;
  const int E = J.n_edges;
  float* pmf = J.pmf + (int64_t)view * E;
  float* cdf = J.cdf + (int64_t)view * (E + 1);
  __shared__ float s_run;
  const int n_chunks = (E + CDF_CHUNK - 1) / CDF_CHUNK;
  if (tid == 0) {
    s_run = 0.0f;
    cdf[0] = 0.0f;
  }
  for (int j = tid; j < min(CDF_CHUNK, E); j += CDF_THREADS) sbuf[j] = pmf[j];
  __syncthreads();
  for (int c = 0; c < n_chunks; c++) {
    if (tid == 0) {
      // 16 values per step in four 16-byte loads; the next 16 are loaded
      // while the current ones are added (the 16 dependent additions outlast
      // a shared-memory load), so only the additions are on the chain
      float* buf = sbuf + (c % 3) * CDF_CHUNK;
      float4* b4 = reinterpret_cast<float4*>(buf);
      const int n = min(CDF_CHUNK, E - c * CDF_CHUNK);
      const int n16 = n & ~15;
      float run = s_run;
      float4 q[4];
#pragma unroll
      for (int k = 0; k < 4; k++) q[k] = n16 > 0 ? b4[k] : make_float4(0.f, 0.f, 0.f, 0.f);
      for (int j = 0; j < n16; j += 16) {
        float4 nq[4];
        const bool more = j + 16 < n16;
#pragma unroll
        for (int k = 0; k < 4; k++) nq[k] = more ? b4[(j >> 2) + 4 + k] : q[k];
#pragma unroll
        for (int k = 0; k < 4; k++) {
          float4 r;
          run = q[k].x + run; r.x = run;
          run = q[k].y + run; r.y = run;
          run = q[k].z + run; r.z = run;
          run = q[k].w + run; r.w = run;
          b4[(j >> 2) + k] = r;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) q[k] = nq[k];
      }
      for (int j = n16; j < n; j++) {
        run = buf[j] + run;
        buf[j] = run;
      }
      s_run = run;
    } else if (tid >= 32) {
      const int t = tid - 32, T = CDF_THREADS - 32;
      if (c >= 1) {  // chunk c-1 is complete (and full: only the last chunk is short)
        const float* done = sbuf + ((c - 1) % 3) * CDF_CHUNK;
        for (int j = t; j < CDF_CHUNK; j += T) cdf[(c - 1) * CDF_CHUNK + j + 1] = done[j];
      }
      if (c + 1 < n_chunks) {
        float* next = sbuf + ((c + 1) % 3) * CDF_CHUNK;
        const int n1 = min(CDF_CHUNK, E - (c + 1) * CDF_CHUNK);
        for (int j = t; j < n1; j += T) next[j] = pmf[(c + 1) * CDF_CHUNK + j];
      }
    }
    __syncthreads();
  }
  if (n_chunks > 0) {
    const int c = n_chunks - 1;
    const float* done = sbuf + (c % 3) * CDF_CHUNK;
    for (int j = tid; j < E - c * CDF_CHUNK; j += CDF_THREADS) cdf[c * CDF_CHUNK + j + 1] = done[j];
  }
  __syncthreads();
  const float total = s_run;
  for (int k = tid; k < E; k += CDF_THREADS) pmf[k] = pmf[k] / total;
  for (int k = tid; k <= E; k += CDF_THREADS) cdf[k] = cdf[k] / total;
}

__device__ __forceinline__ int upper_bound_idx(const float* cdf, int n, float u) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (u < cdf[mid]) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Sample i of a view: edge choice and rejection (drender.h:326-345).
__device__ __forceinline__ bool edge_select_test(const JobDev& J, int view, int i, int& edge_id) {
  edge_id = 0;
  if (i >= J.edge_samples || J.n_edges <= 0) return false;
  const float rnd0 = __ldg(J.rnd + 2 * i), rnd1 = __ldg(J.rnd + 2 * i + 1);
  const float* cdf = J.cdf + (int64_t)view * (J.n_edges + 1);
  edge_id = clampi(upper_bound_idx(cdf, J.n_edges + 1, rnd0) - 1, 0, J.n_edges - 1);
  // silhouette mode: a view without silhouette edges has no samples
  if (J.edge_sil && !(J.pmf[(int64_t)view * J.n_edges + edge_id] > 0.0f)) return false;
  const int4 ed = __ldg(J.edges + edge_id);
  const float4* P = J.proj + (int64_t)view * J.n_vertices;
  const float4 a = P[ed.x], b = P[ed.y];
  const float t = rnd1;
  const float px = a.x + t * (b.x - a.x), py = a.y + t * (b.y - a.y);
  const int xi = (int)px, yi = (int)py;
  if (xi < 0 || yi < 0 || xi >= J.W || yi >= J.H) return false;
  const float4 ad = J.adj[(int64_t)view * J.W * J.H + (int64_t)yi * J.W + xi];
  return !(length(mk(ad.x, ad.y, ad.z)) < 1e-3f);
}

// Warp-aggregated append (all 32 lanes call it).
__device__ __forceinline__ void queue_append(int4* queue, int* count, int cap, bool keep, int4 entry) {
  const unsigned ballot = __ballot_sync(0xffffffffu, keep);
  if (!ballot) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(ballot) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(ballot));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (keep) {
    const int slot = base + __popc(ballot & ((1u << lane) - 1u));
    if (slot < cap) queue[slot] = entry;
  }
}

// One shading point of an edge sample: the generic shader (every model), or
// the model MODE alone.
template <int MODE>
__device__ __forceinline__ f3 edge_point(const JobDev& J, const CamDev& cam, float x, float y, uint32_t key,
                                         int view) {
  if (MODE == 0) return shade_generic(J, cam, x, y, key, view);
  return shade_p<MODE, false>(J, cam, x, y, key, true, nullptr, false, float4{0.0f, 0.0f, 0.0f, 0.0f}, view);
}

// Shading and chain rule of queue entries [q0, q0+32) (one per lane).  DET:
// the deterministic-mode variant (records for jobs that have record buffers).
// PAIRS: two lanes per entry, the even one shading the inside point and the
// odd one the outside point in the same traversal call (16 entries per
// warp); else one lane per entry shades both points in turn.
template <bool DET, bool PAIRS = false, int MODE = 0>
__device__ __forceinline__ void edge_shade_warp(const JobDev* jobs, const int4* queue, int n, int q0,
                                                const int* order = nullptr) {
  const int lane = threadIdx.x & 31;
  const int side = PAIRS ? (lane & 1) : 0;
  const int q = PAIRS ? q0 + (lane >> 1) : q0 + lane;
  float tr[12];
#pragma unroll
  for (int k = 0; k < 12; k++) tr[k] = 0.0f;
  float* target = nullptr;  // transform-gradient block this lane adds to
  if (q < n) {
    const int4 it = queue[order ? order[q] : q];
    const int view = it.x, i = it.y, edge_id = it.z;
    const JobDev& J = jobs[it.w];
    const CamDev& cam = J.cams[view];
    const int4 ed = __ldg(J.edges + edge_id);
    const int2 mi = __ldg(J.edge_mi + edge_id);
    const float pm = J.pmf[(int64_t)view * J.n_edges + edge_id];
    const float4* P = J.proj + (int64_t)view * J.n_vertices;
    const float4 pa = P[ed.x], pb = P[ed.y];
    const float t = __ldg(J.rnd + 2 * i + 1);
    const float dx0 = pb.x - pa.x, dy0 = pb.y - pa.y;
    const float px = pa.x + t * dx0, py = pa.y + t * dy0;
    const int xi = (int)px, yi = (int)py;
    const float4 ad = J.adj[(int64_t)view * J.W * J.H + (int64_t)yi * J.W + xi];
    const float dl = sqrtf(dx0 * dx0 + dy0 * dy0);
    const float nx = -(dy0 / dl), ny = dx0 / dl;  // normal2D of the unit edge direction
    const float cinx = px - 1e-3f * nx, ciny = py - 1e-3f * ny;
    const float coutx = px + 1e-3f * nx, couty = py + 1e-3f * ny;
    const uint32_t key_in = 0xA511E9B3u ^ ((uint32_t)(i * 2u) * 2654435761u);
    const uint32_t key_out = 0xA511E9B3u ^ ((uint32_t)(i * 2u + 1u) * 2654435761u);
    f3 color_in, color_out;
    if (PAIRS) {
      const f3 mine = edge_point<MODE>(J, cam, side ? coutx : cinx, side ? couty : ciny, side ? key_out : key_in, view);
      const unsigned pair = 3u << (lane & ~1);  // both lanes of an entry take this branch
      const f3 other = mk(__shfl_xor_sync(pair, mine.x, 1), __shfl_xor_sync(pair, mine.y, 1),
                          __shfl_xor_sync(pair, mine.z, 1));
      color_in = side ? other : mine;
      color_out = side ? mine : other;
    } else {
      color_in = edge_point<MODE>(J, cam, cinx, ciny, key_in, view);
      color_out = edge_point<MODE>(J, cam, coutx, couty, key_out, view);
    }
    const float pdf = pm / sqrtf(dx0 * dx0 + dy0 * dy0);
    const float weight = 1.0f / (pdf * (float)J.edge_samples);
    const float adjv = dot(color_in - color_out, mk(ad.x, ad.y, ad.z));
    if (side == 0 && adjv * adjv > 0.0f) {  // (PAIRS: the even lane applies the chain rule)
      const float d0x = (1 - t) * nx * adjv * weight, d0y = (1 - t) * ny * adjv * weight;
      const float d1x = t * nx * adjv * weight, d1y = t * ny * adjv * weight;
      const f3 v0 = ld3(J.pos, ed.x), v1 = ld3(J.pos, ed.y);
      const f3 g0x = vs_grad(cam, v0, false), g0y = vs_grad(cam, v0, true);
      const f3 g1x = vs_grad(cam, v1, false), g1y = vs_grad(cam, v1, true);
      // world-space gradient of the two endpoints: the reference keeps dx/dX
      // and dy/dY only for the x and y components (drender.cpp:45-51); the
      // exact form is the full (dx,dy)/(X,Y,Z) Jacobian transposed
      const bool exact = J.edge_exact;
      const float dv0_dx = exact ? g0x.x * d0x + g0y.x * d0y : g0x.x * d0x;
      const float dv0_dy = exact ? g0x.y * d0x + g0y.y * d0y : g0y.y * d0y;
      const float dv0_dz = (g0x.z * d0x + g0y.z * d0y);
      const float dv1_dx = exact ? g1x.x * d1x + g1y.x * d1y : g1x.x * d1x;
      const float dv1_dy = exact ? g1x.y * d1x + g1y.y * d1y : g1y.y * d1y;
      const float dv1_dz = (g1x.z * d1x + g1y.z * d1y);
      const MeshDev& md = J.meshes[mi.x];
      if (md.dslot >= 0) {
        float* g = J.grad + md.g_base + md.pos_off;
        f3 d0, d1;
        if (exact) {
          // to mesh-local positions: the transpose of the edge's own instance
          // transform (world = T * local)
          const float* T = J.block_tr + 32 * (md.block0 + mi.y);
          d0 = mk(T[0] * dv0_dx + T[1] * dv0_dy + T[2] * dv0_dz, T[4] * dv0_dx + T[5] * dv0_dy + T[6] * dv0_dz,
                  T[8] * dv0_dx + T[9] * dv0_dy + T[10] * dv0_dz);
          d1 = mk(T[0] * dv1_dx + T[1] * dv1_dy + T[2] * dv1_dz, T[4] * dv1_dx + T[5] * dv1_dy + T[6] * dv1_dz,
                  T[8] * dv1_dx + T[9] * dv1_dy + T[10] * dv1_dz);
        } else {
          const float* M = J.tr_inv0 + 16 * mi.y;  // get_transform_inv(0)[inst]
          d0 = mk(M[0] * dv0_dx + M[4] * dv0_dy + M[8] * dv0_dz, M[1] * dv0_dx + M[5] * dv0_dy + M[9] * dv0_dz,
                  M[2] * dv0_dx + M[6] * dv0_dy + M[10] * dv0_dz);
          d1 = mk(M[0] * dv1_dx + M[4] * dv1_dy + M[8] * dv1_dz, M[1] * dv1_dx + M[5] * dv1_dy + M[9] * dv1_dz,
                  M[2] * dv1_dx + M[6] * dv1_dy + M[10] * dv1_dz);
        }
        if (!(DET && J.det)) {
          atomicAdd(g + ed.z * 3 + 0, d0.x);
          atomicAdd(g + ed.z * 3 + 1, d0.y);
          atomicAdd(g + ed.z * 3 + 2, d0.z);
          atomicAdd(g + ed.w * 3 + 0, d1.x);
          atomicAdd(g + ed.w * 3 + 1, d1.y);
          atomicAdd(g + ed.w * 3 + 2, d1.z);
        }
        const f3 o0 = ld3(J.orig, ed.x), o1 = ld3(J.orig, ed.y);
        tr[0] = o0.x * dv0_dx + o1.x * dv1_dx;
        tr[1] = o0.y * dv0_dx + o1.y * dv1_dx;
        tr[2] = o0.z * dv0_dx + o1.z * dv1_dx;
        tr[3] = 1 * dv0_dx + 1 * dv1_dx;
        tr[4] = o0.x * dv0_dy + o1.x * dv1_dy;
        tr[5] = o0.y * dv0_dy + o1.y * dv1_dy;
        tr[6] = o0.z * dv0_dy + o1.z * dv1_dy;
        tr[7] = 1 * dv0_dy + 1 * dv1_dy;
        tr[8] = o0.x * dv0_dz + o1.x * dv1_dz;
        tr[9] = o0.y * dv0_dz + o1.y * dv1_dz;
        tr[10] = o0.z * dv0_dz + o1.z * dv1_dz;
        tr[11] = 1 * dv0_dz + 1 * dv1_dz;
        target = J.grad + md.g_base + md.tr_off + 12 * mi.y;
        if (DET && J.det) {
          // the records in the sample's own slots, in a fixed order
          const int64_t slot = edge_rec_slot(J, view, i);
          const uint32_t kp = (uint32_t)(g - J.grad), kt = (uint32_t)(target - J.grad);
          J.rec_key[slot + 0] = kp + 3 * ed.z;
          J.rec_val[slot + 0] = make_float4(d0.x, d0.y, d0.z, 0.0f);
          J.rec_key[slot + 1] = kp + 3 * ed.w;
          J.rec_val[slot + 1] = make_float4(d1.x, d1.y, d1.z, 0.0f);
          if (J.det_tr) {
            // the job's only transform block: 12 dense values per sample,
            // summed later in a fixed order without sorting
            float4* T = reinterpret_cast<float4*>(J.det_tr + ((int64_t)view * J.edge_samples + i) * 12);
#pragma unroll
            for (int k = 0; k < 3; k++) T[k] = make_float4(tr[4 * k], tr[4 * k + 1], tr[4 * k + 2], tr[4 * k + 3]);
            J.rec_count[edge_region(J, view, i)] = 2;
          } else {
#pragma unroll
            for (int k = 0; k < 4; k++) {
              J.rec_key[slot + 2 + k] = kt + 3 * k;
              J.rec_val[slot + 2 + k] = make_float4(tr[3 * k], tr[3 * k + 1], tr[3 * k + 2], 0.0f);
            }
            J.rec_count[edge_region(J, view, i)] = kEdgeRecords;
          }
          target = nullptr;
        }
      }
    }
  }
  // transform gradient: one atomic per warp when every contributing lane
  // targets the same block, per lane otherwise
  const unsigned any = __ballot_sync(0xffffffffu, target != nullptr);
  if (!any) return;
  const unsigned long long mine = (unsigned long long)target;
  const unsigned long long lead = __shfl_sync(0xffffffffu, mine, __ffs(any) - 1);
  const bool uniform = __all_sync(0xffffffffu, target == nullptr || mine == lead);
  if (uniform) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      float v = tr[k];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      tr[k] = v;
    }
    if (lane == 0)
      for (int k = 0; k < 12; k++) atomicAdd(reinterpret_cast<float*>(lead) + k, tr[k]);
  } else if (target) {
    for (int k = 0; k < 12; k++) atomicAdd(target + k, tr[k]);
  }
}

// ---- single job: blockIdx.y = view -----------------------------------------
__global__ void k_edge_project(const JobDev* jobs, int job) {
  const JobDev& J = jobs[job];
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < J.n_vertices) edge_project_body(J, blockIdx.y, v);
}

__global__ void k_edge_pmf(const JobDev* jobs, int job) {
  const JobDev& J = jobs[job];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < J.n_edges) edge_pmf_body(J, blockIdx.y, e);
}

__global__ void __launch_bounds__(CDF_THREADS) k_edge_cdf(const JobDev* jobs, int job) {
  __shared__ __align__(16) float sbuf[CDF_SMEM];
  edge_cdf_body(jobs[job], blockIdx.x, sbuf);
}

// Samples are taken in rnd_order when the job has it (consecutive entries
// then fall on the same or neighbouring edges, the order the shading pass
// wants) and in index order otherwise.
__global__ void k_edge_select(const JobDev* jobs, int job) {
  const JobDev& J = jobs[job];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = J.rnd_order && j < J.edge_samples ? __ldg(J.rnd_order + j) : j;
  const int view = blockIdx.y;
  int edge_id;
  const bool keep = edge_select_test(J, view, i, edge_id);
  queue_append(J.queue, J.queue_count, J.queue_cap, keep, make_int4(view, i, edge_id, job));
}

// Four resident blocks per SM (64 registers, with spills): faster on GB300
// than two or three, for the point-light and path models alike.
#ifndef DRGB_EDGE_MIN_BLOCKS
#define DRGB_EDGE_MIN_BLOCKS 4
#endif
// Persistent over the queue, in whole warps (the reductions need every lane):
// each warp takes the next 32 entries from a counter (count[1], zeroed with
// the queue count), so warps that drew cheap samples take more and the launch
// ends without a tail of idle SMs; -DDRGB_EDGE_STATIC strides statically.
// `order` (may be null) is the shading order of the entries.
template <bool DET, bool PAIRS = false, int MODE = 0>
__device__ __forceinline__ void edge_shade_loop(const JobDev* jobs, const int4* queue, int n, int* work,
                                                const int* order) {
  constexpr int kPerWarp = PAIRS ? 16 : 32;
#ifdef DRGB_EDGE_STATIC
  (void)work;
  const int stride = gridDim.x * blockDim.x / 32 * kPerWarp;
  for (int q0 = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * kPerWarp; q0 < n; q0 += stride)
    edge_shade_warp<DET, PAIRS, MODE>(jobs, queue, n, q0, order);
#else
  const int lane = threadIdx.x & 31;
  while (true) {
    int q0 = 0;
    if (lane == 0) q0 = atomicAdd(work, kPerWarp);
    q0 = __shfl_sync(0xffffffffu, q0, 0);
    if (q0 >= n) break;
    edge_shade_warp<DET, PAIRS, MODE>(jobs, queue, n, q0, order);
  }
#endif
}

template <bool DET>
__global__ void __launch_bounds__(256, DRGB_EDGE_MIN_BLOCKS) k_edge_shade_q(const JobDev* jobs, const int4* queue, int* count,
                                                      int cap, const int* order) {
  edge_shade_loop<DET>(jobs, queue, min(count[0], cap), count + 1, order);
}

// Sort keys of a batch queue: each job's (view, edge) range starts at the
// job's edge_key_base.
__global__ void k_b_queue_keys(const JobDev* jobs, const int4* queue, const int* count, int cap, uint32_t* keys,
                               int* idx, int* n_out) {
  const int n = min(*count, cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) *n_out = n;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int4 e = queue[q];
    const JobDev& J = jobs[e.w];
    keys[q] = J.edge_key_base + (uint32_t)e.x * (uint32_t)J.n_edges + (uint32_t)e.z;
    idx[q] = q;
  }
}

// Single job: the queue, its counter and its capacity are the job's own;
// `order` (may be null) is the shading order of the queue entries.
// MODE != 0: the shader of that model alone (the point-light model of the
// benchmark; fewer registers and spills than the generic shader).
template <bool DET, bool PAIRS, int MODE = 0>
__global__ void __launch_bounds__(256, DRGB_EDGE_MIN_BLOCKS) k_edge_shade_job(const JobDev* jobs, int job,
                                                                              const int* order) {
  const JobDev& J = jobs[job];
  stage_top_nodes(J);
  edge_shade_loop<DET, PAIRS, MODE>(jobs, J.queue, min(J.queue_count[0], J.queue_cap), J.queue_count + 1, order);
}

// Lane pairs for the path model, whose two points cost alike but vary a lot
// from sample to sample (GB300, 200k-triangle stress workload: edge pass
// 4.34 -> 4.03 ms); one lane per entry for the others, where the inside point
// of a silhouette sample hits and casts a shadow ray and the outside point
// misses (point-light icosphere: 1.50 ms against 2.10 ms with pairs).
#ifdef DRGB_EDGE_GENERIC
constexpr bool kEdgeSpecialised = false;
#else
constexpr bool kEdgeSpecialised = true;
#endif
static void launch_shade_job(const JobDev* d_jobs, int job, int mode, int grid, const int* order, bool det,
                             cudaStream_t s) {
  grid = std::max(1, grid);
  const bool pairs = model_is_path(mode);
  if (det) {
    if (pairs) k_edge_shade_job<true, true><<<grid, 256, 0, s>>>(d_jobs, job, order);
    else k_edge_shade_job<true, false><<<grid, 256, 0, s>>>(d_jobs, job, order);
  } else if (pairs) {
    k_edge_shade_job<false, true><<<grid, 256, 0, s>>>(d_jobs, job, order);
  } else if (mode == LAMBERT_POINT_VCOLOR && kEdgeSpecialised) {
    k_edge_shade_job<false, false, LAMBERT_POINT_VCOLOR><<<grid, 256, 0, s>>>(d_jobs, job, order);
  } else {
    k_edge_shade_job<false, false><<<grid, 256, 0, s>>>(d_jobs, job, order);
  }
}

// Sort keys of the queue entries: (view, edge), so that neighbouring lanes
// shade points of the same edge (coherent rays); the value is the entry.
__global__ void k_queue_keys(const JobDev* jobs, int job, uint32_t* keys, int* idx, int* n_out) {
  const JobDev& J = jobs[job];
  const int n = min(*J.queue_count, J.queue_cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) *n_out = n;  // the sort's count, within the buffers
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int4 e = J.queue[q];
    keys[q] = (uint32_t)e.x * (uint32_t)J.n_edges + (uint32_t)e.z;
    idx[q] = q;
  }
}

// ---- batched: segment tables over (job, view) pairs --------------------------
__global__ void k_b_edge_project(const JobDev* jobs, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int v = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (v < sg.count) edge_project_body(jobs[sg.job], sg.sub, v);
}

__global__ void k_b_edge_pmf(const JobDev* jobs, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int e = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (e < sg.count) edge_pmf_body(jobs[sg.job], sg.sub, e);
}

// one block per (job, view) pair: pairs[b].job / .sub
__global__ void __launch_bounds__(CDF_THREADS) k_b_edge_cdf(const JobDev* jobs, const Seg* pairs, int n_pairs) {
  __shared__ __align__(16) float sbuf[CDF_SMEM];
  if ((int)blockIdx.x >= n_pairs) return;
  const Seg sg = pairs[blockIdx.x];
  edge_cdf_body(jobs[sg.job], sg.sub, sbuf);
}

__global__ void k_b_edge_select(const JobDev* jobs, const Seg* segs, int nseg, int4* queue, int* count, int cap) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int i = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  int edge_id = 0;
  const bool keep = i < sg.count && edge_select_test(jobs[sg.job], sg.sub, i, edge_id);
  queue_append(queue, count, cap, keep, make_int4(sg.sub, i, edge_id, sg.job));
}

// Same launch sequence with every size and the sample-queue counter passed
// explicitly (for callers whose buffers are not owned by a Job).
// The queue's shading order sorted by (view, edge); null when not sorted.
// (+25 % on the edge pass of the point-light workload on GB300; builds
// with -DDRGB_EDGE_NO_SORT shade in queue order.)
static const int* sort_queue(const JobDev* d_jobs, int job, const Job& J, int grid, cudaStream_t s) {
#ifndef DRGB_EDGE_NO_SORT
  // samples selected in rnd_order are already grouped by edge within a view
  if (!J.qkey[0].p || J.n_edges <= 0 || J.dev.rnd_order) return nullptr;
  k_queue_keys<<<std::max(1, grid), 256, 0, s>>>(d_jobs, job, J.qkey[0].p, J.qidx[0].p, J.qn.p);
  count_launch();
  uint64_t top = (uint64_t)J.n_views * (uint64_t)J.n_edges;
  int bits = 1;
  while (bits < 32 && (1ull << bits) < top) bits++;
  uint32_t* keys[2] = {J.qkey[0].p, J.qkey[1].p};
  int* vals[2] = {J.qidx[0].p, J.qidx[1].p};
  return vals[sort_pairs_device(keys, vals, J.qn.p, bits, J.qhist.p, s)];
#else
  (void)d_jobs; (void)job; (void)J; (void)grid; (void)s;
  return nullptr;
#endif
}

// Jq (may be null): the job whose queue-sort buffers order the shading.
// The part of the edge pass that needs only the vertices: projection, pmf
// and CDF of every view (may run beside the pixel pass).
void launch_edges_prep(const JobDev* d_jobs, int job, int n_edges, int n_views, int n_vertices, cudaStream_t s) {
  if (n_edges <= 0 || n_views <= 0) return;
  k_edge_project<<<dim3((n_vertices + 255) / 256, n_views), 256, 0, s>>>(d_jobs, job);
  k_edge_pmf<<<dim3((n_edges + 255) / 256, n_views), 256, 0, s>>>(d_jobs, job);
  k_edge_cdf<<<n_views, CDF_THREADS, 0, s>>>(d_jobs, job);
  count_launch(3);
}

// The rest, which reads the adjoint image: selection, ordering, shading.
void launch_edges_rest(const JobDev* d_jobs, int job, int n_edges, int n_views, int edge_samples, int* queue_count,
                       int shade_grid, cudaStream_t s, bool det, const Job* Jq, int mode) {
  if (n_edges <= 0 || n_views <= 0 || edge_samples <= 0) return;
  DRGB_CUDA(cudaMemsetAsync(queue_count, 0, 2 * sizeof(int), s));  // queue count, shading counter
  k_edge_select<<<dim3((edge_samples + 255) / 256, n_views), 256, 0, s>>>(d_jobs, job);
  const int* order = Jq ? sort_queue(d_jobs, job, *Jq, shade_grid, s) : nullptr;
  launch_shade_job(d_jobs, job, mode, shade_grid, order, det, s);
  count_launch(2);
}

void launch_edges_raw(const JobDev* d_jobs, int job, int n_edges, int n_views, int n_vertices, int edge_samples,
                      int* queue_count, int shade_grid, cudaStream_t s, bool det, const Job* Jq, int mode) {
  if (n_edges <= 0 || n_views <= 0 || edge_samples <= 0) return;
  k_edge_project<<<dim3((n_vertices + 255) / 256, n_views), 256, 0, s>>>(d_jobs, job);
  k_edge_pmf<<<dim3((n_edges + 255) / 256, n_views), 256, 0, s>>>(d_jobs, job);
  k_edge_cdf<<<n_views, CDF_THREADS, 0, s>>>(d_jobs, job);
  DRGB_CUDA(cudaMemsetAsync(queue_count, 0, 2 * sizeof(int), s));  // queue count, shading counter
  k_edge_select<<<dim3((edge_samples + 255) / 256, n_views), 256, 0, s>>>(d_jobs, job);
  // the queue, its counter and capacity are read from the job on the device
  const int* order = Jq ? sort_queue(d_jobs, job, *Jq, shade_grid, s) : nullptr;
  launch_shade_job(d_jobs, job, mode, shade_grid, order, det, s);
  count_launch(5);
}

void launch_edges(const JobDev* d_jobs, int job, const Job& J, int shade_grid, cudaStream_t s) {
  if (J.n_edges <= 0 || J.n_views <= 0) return;
  launch_edges_raw(d_jobs, job, J.n_edges, J.n_views, J.n_vertices, J.dev.edge_samples, J.queue_count.p, shade_grid,
                   s, J.det != 0, &J, J.mode);
}

// Edge pass of every job of a batch; the shared queue holds (view, sample,
// edge, job) entries of all jobs.
void launch_b_edges(const JobDev* d_jobs, const Seg* proj_segs, int n_proj, int proj_chunks, const Seg* pmf_segs,
                    int n_pmf, int pmf_chunks, const Seg* pairs, int n_pairs, const Seg* sel_segs, int n_sel,
                    int sel_chunks, int4* queue, int* count, int cap, int shade_grid, cudaStream_t s, bool det,
                    const QueueSort* qs) {
  if (n_pairs <= 0) return;
  if (proj_chunks > 0) k_b_edge_project<<<proj_chunks, 256, 0, s>>>(d_jobs, proj_segs, n_proj);
  if (pmf_chunks > 0) k_b_edge_pmf<<<pmf_chunks, 256, 0, s>>>(d_jobs, pmf_segs, n_pmf);
  k_b_edge_cdf<<<n_pairs, CDF_THREADS, 0, s>>>(d_jobs, pairs, n_pairs);
  DRGB_CUDA(cudaMemsetAsync(count, 0, 2 * sizeof(int), s));  // queue count, shading counter
  if (sel_chunks > 0) k_b_edge_select<<<sel_chunks, 256, 0, s>>>(d_jobs, sel_segs, n_sel, queue, count, cap);
  const int* order = nullptr;
#ifndef DRGB_EDGE_NO_SORT
  if (qs && qs->keys[0]) {
    k_b_queue_keys<<<std::max(1, shade_grid), 256, 0, s>>>(d_jobs, queue, count, cap, qs->keys[0], qs->vals[0], qs->n);
    count_launch();
    uint32_t* keys[2] = {qs->keys[0], qs->keys[1]};
    int* vals[2] = {qs->vals[0], qs->vals[1]};
    order = vals[sort_pairs_device(keys, vals, qs->n, qs->bits, qs->hist, s)];
  }
#endif
  if (det) k_edge_shade_q<true><<<std::max(1, shade_grid), 256, 0, s>>>(d_jobs, queue, count, cap, order);
  else k_edge_shade_q<false><<<std::max(1, shade_grid), 256, 0, s>>>(d_jobs, queue, count, cap, order);
  count_launch(5);
}

}  // namespace drgb
