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

// Warp-aggregated scatter of per-vertex colour gradients.  All 32 lanes
// must call it; lanes without a contribution pass tri = -1.
__device__ __forceinline__ void scatter_vertex_colors(const JobDev& J, int tri, int gA, int gB, int gC,
                                                      const float c[9], float* wscr) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(0xffffffffu, tri);
  const int leader = __ffs(peers) - 1;
#pragma unroll
  for (int i = 0; i < 9; i++) wscr[i * 32 + lane] = c[i];
  __syncwarp();
  if (tri >= 0 && lane == leader) {
    float s[9];
#pragma unroll
    for (int i = 0; i < 9; i++) s[i] = 0.0f;
    unsigned m = peers;
    while (m) {
      const int l = __ffs(m) - 1;
      m &= m - 1;
#pragma unroll
      for (int i = 0; i < 9; i++) s[i] += wscr[i * 32 + l];
    }
    const int b = __ldg(J.tri_v + tri).w;
    const BlockDev bd = J.blocks[b];
    const MeshDev& md = J.meshes[bd.mesh];
    if (md.dslot >= 0) {
      float* g = J.grad + md.g_base + md.color_off;
      const int a = gA - bd.vert_off, bb = gB - bd.vert_off, cc = gC - bd.vert_off;
      atomicAdd(g + 3 * a + 0, s[0]); atomicAdd(g + 3 * a + 1, s[1]); atomicAdd(g + 3 * a + 2, s[2]);
      atomicAdd(g + 3 * bb + 0, s[3]); atomicAdd(g + 3 * bb + 1, s[4]); atomicAdd(g + 3 * bb + 2, s[5]);
      atomicAdd(g + 3 * cc + 0, s[6]); atomicAdd(g + 3 * cc + 1, s[7]); atomicAdd(g + 3 * cc + 2, s[8]);
    }
  }
  __syncwarp();
}

// sample_bilinear_clamp_3f_grad (shade_common.cpp:23-46), atomics.
__device__ __forceinline__ void texture_grad(f3 val, float tx, float ty, int w, int h, float* data) {
  const float px = tx * (float)w, py = ty * (float)h;
  const int ix = (int)px, iy = (int)py;
  const int x0 = clampi(ix, 0, w - 1), y0 = clampi(iy, 0, h - 1);
  const int x1 = clampi(ix + 1, 0, w - 1), y1 = clampi(iy + 1, 0, h - 1);
  const float dx = px - (float)x0, dy = py - (float)y0;
  float* d00 = data + 3 * (y0 * w + x0);
  float* d01 = data + 3 * (y1 * w + x0);
  float* d10 = data + 3 * (y0 * w + x1);
  float* d11 = data + 3 * (y1 * w + x1);
  const float w00 = (1 - dx) * (1 - dy), w01 = (1 - dx) * dy, w10 = dx * (1 - dy), w11 = dx * dy;
  atomicAdd(d00 + 0, w00 * val.x); atomicAdd(d00 + 1, w00 * val.y); atomicAdd(d00 + 2, w00 * val.z);
  atomicAdd(d01 + 0, w01 * val.x); atomicAdd(d01 + 1, w01 * val.y); atomicAdd(d01 + 2, w01 * val.z);
  atomicAdd(d10 + 0, w10 * val.x); atomicAdd(d10 + 1, w10 * val.y); atomicAdd(d10 + 2, w10 * val.z);
  atomicAdd(d11 + 0, w11 * val.x); atomicAdd(d11 + 1, w11 * val.y); atomicAdd(d11 + 2, w11 * val.z);
}

// shade_grad<M> for one sample; every lane of the warp must call it.
__device__ __forceinline__ void shade_grad(const JobDev& J, const CamDev& cam, bool active, float x, float y, f3 val,
                                           uint32_t key, float* wscr) {
  Surf s;
  bool hit = false;
  if (active) hit = cast(J, cam, x, y, s);
  if (model_has_color(J.mode)) {
    float c[9];
    int tri = -1, gA = 0, gB = 0, gC = 0;
#pragma unroll
    for (int i = 0; i < 9; i++) c[i] = 0.0f;
    if (hit) {
      const float u = s.h.u, v = s.h.v;
      f3 ca, cb, cc;
      if (J.mode == VERTEX_COLOR) {
        ca = val * (1.0f - u - v);
        cb = val * v;
        cc = val * u;
      } else if (J.mode == LAMBERT_POINT_VCOLOR) {
        const float k = lpv_factor(J, s);
        ca = val * ((1.0f - u - v) * k);
        cb = val * (v * k);
        cc = val * (u * k);
      } else {
        f3 d0;
        path_diffuse(J, s, key, &d0);
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
    scatter_vertex_colors(J, tri, gA, gB, gC, c, wscr);
  } else if (model_has_tex(J.mode) && hit) {
    const BlockDev bd = J.blocks[s.block];
    const MeshDev& md = J.meshes[bd.mesh];
    if (md.dslot >= 0 && md.tex_off >= 0) {
      const float2 tc = interp_tc(J, s);
      texture_grad(val, tc.x, tc.y, md.tex_w, md.tex_h, J.grad + md.g_base + md.tex_off);
    }
  }
}

template <int FLAGS>
__global__ void __launch_bounds__(PX_THREADS) k_pixels(const JobDev* __restrict__ jobs, const int4* __restrict__ items,
                                                       int n_items, int* counter) {
  __shared__ JobDev sJ;
  __shared__ CamDev sC;
  __shared__ float s_col[PX_THREADS * 3];
  __shared__ float4 s_adj[PX_THREADS];
  __shared__ double s_loss[PX_THREADS];
  __shared__ float s_ham[2 * 64];
  __shared__ float wscr_all[PX_THREADS / 32][9 * 32];
  __shared__ int s_item;
  __shared__ int s_job;
  const int tid = threadIdx.x;
  float* wscr = wscr_all[tid >> 5];
  if (tid == 0) s_job = -1;
  __syncthreads();
  for (;;) {
    if (tid == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) break;
    const int4 item = items[it];
    if (item.x != s_job) {
      const int* src = reinterpret_cast<const int*>(jobs + item.x);
      int* dst = reinterpret_cast<int*>(&sJ);
      for (int i = tid; i < (int)(sizeof(JobDev) / sizeof(int)); i += PX_THREADS) dst[i] = src[i];
      __syncthreads();
      for (int i = tid; i < 2 * sJ.spp && i < 128; i += PX_THREADS) s_ham[i] = sJ.ham[i];
      if (tid == 0) s_job = item.x;
    }
    {
      const int* src = reinterpret_cast<const int*>(sJ.cams + item.y);
      int* dst = reinterpret_cast<int*>(&sC);
      for (int i = tid; i < (int)(sizeof(CamDev) / sizeof(int)); i += PX_THREADS) dst[i] = src[i];
    }
    __syncthreads();
    const JobDev& J = sJ;
    const int view = item.y, x0 = item.z, y0 = item.w;
    const int W = (int)sC.width, H = (int)sC.height;
    const int tw = J.tile_w, th = J.tile_h;
    const int P = tw * th;
    const int S = J.S, sq = J.sq;
    const int NS = P * S;
    // sample of this thread (samples of a pixel are consecutive threads)
    const int p = tid / S, k = tid - p * S;
    const int px = x0 + p % tw, py = y0 + p / tw;
    const bool valid = tid < NS && px < W && py < H;
    const int64_t pix = valid ? (int64_t)py * W + px : 0;
    if (FLAGS & PX_FWD) {
      f3 c = mk(0.0f, 0.0f, 0.0f);
      if (valid) {
        const int dy = k / sq, dx = k - dy * sq;
        const float xoff = (dx + 0.5f) / (float)sq;
        const float yoff = (dy + 0.5f) / (float)sq;
        const uint32_t key = ((uint32_t)view * 0x9E3779B9u) ^
                             ((uint32_t)(pix * 64 + dy * sq + dx) * 2654435761u);
        c = shade(J, sC, (float)px + xoff, (float)py + yoff, key) / (float)S;
      }
      if (tid < NS) {
        s_col[3 * tid + 0] = c.x;
        s_col[3 * tid + 1] = c.y;
        s_col[3 * tid + 2] = c.z;
      }
      __syncthreads();
      double lsum = 0.0;
      if (tid < P) {
        const int qx = x0 + tid % tw, qy = y0 + tid / tw;
        if (qx < W && qy < H) {
          float ax = 0.0f, ay = 0.0f, az = 0.0f;
          for (int j = 0; j < S; j++) {
            ax += s_col[3 * (tid * S + j) + 0];
            ay += s_col[3 * (tid * S + j) + 1];
            az += s_col[3 * (tid * S + j) + 2];
          }
          const int64_t q = (int64_t)qy * W + qx;
          if ((FLAGS & PX_IMG) && J.images) {
            float* o = J.images + 3 * (J.img_off[view] + q);
            o[0] = ax; o[1] = ay; o[2] = az;
          }
          if (FLAGS & PX_LOSS) {
            const float* t = J.targets + 3 * (J.img_off[view] + q);
            const float dx = ax - t[0], dy = ay - t[1], dz = az - t[2];
            const float4 a = make_float4(2.0f * dx, 2.0f * dy, 2.0f * dz, 0.0f);
            s_adj[tid] = a;
            J.adj[(int64_t)view * J.W * J.H + q] = a;
            lsum = (double)(dx * dx + dy * dy + dz * dz);
          }
        }
        s_loss[tid] = lsum;
      }
      __syncthreads();
      if ((FLAGS & PX_LOSS) && tid == 0) {
        double acc = 0.0;
        for (int j = 0; j < P; j++) acc += s_loss[j];
        J.loss_part[it - J.item_base] = acc;
      }
    }
    if (FLAGS & PX_ADJ) {
      if (!(FLAGS & PX_LOSS)) {
        if (tid < P) {
          const int qx = x0 + tid % tw, qy = y0 + tid / tw;
          float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          if (qx < W && qy < H) {
            const float* src = J.adj_in + 3 * ((int64_t)view * J.W * J.H + (int64_t)qy * W + qx);
            a = make_float4(src[0], src[1], src[2], 0.0f);
          }
          s_adj[tid] = a;
        }
        __syncthreads();
      }
      // each warp runs its samples together (the scatter is warp-collective)
      f3 val = mk(0.0f, 0.0f, 0.0f);
      bool act = false;
      float sx = 0.0f, sy = 0.0f;
      uint32_t key = 0;
      if (valid) {
        const float4 a = s_adj[p];
        val = mk(a.x, a.y, a.z) / (float)S;
        act = !(val.x == 0.0f && val.y == 0.0f && val.z == 0.0f);
        sx = (float)px + s_ham[2 * k];
        sy = (float)py + s_ham[2 * k + 1];
        key = ((uint32_t)view * 0x9E3779B9u) ^ 0x5bd1e995u ^ ((uint32_t)(pix * 64 + k) * 2654435761u);
      }
      shade_grad(J, sC, act, sx, sy, val, key, wscr);
    }
    __syncthreads();
  }
}

// Loss of each job: per view, double sum of its items' partials -> float;
// float sum over views; divided by views*W*H (drender.h:184-190).
__global__ void k_loss_finalize(const JobDev* jobs, int n_jobs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_jobs) return;
  const JobDev& J = jobs[j];
  const int per_view = J.item_count / J.n_views;
  float mse = 0.0f;
  for (int v = 0; v < J.n_views; v++) {
    double acc = 0.0;
    for (int i = 0; i < per_view; i++) acc += J.loss_part[v * per_view + i];
    mse += (float)acc;
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

void launch_pixels(const JobDev* d_jobs, const int4* d_items, int n_items, int* d_counter, int flags, int grid,
                   cudaStream_t s) {
  if (n_items <= 0) return;
  DRGB_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(int), s));
  if (grid <= 0 || grid > n_items) grid = n_items;
  switch (flags) {
    case PX_FWD | PX_IMG:
      k_pixels<PX_FWD | PX_IMG><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter);
      break;
    case PX_FWD | PX_LOSS | PX_ADJ | PX_IMG:
      k_pixels<PX_FWD | PX_LOSS | PX_ADJ | PX_IMG><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter);
      break;
    case PX_FWD | PX_LOSS | PX_ADJ:
      k_pixels<PX_FWD | PX_LOSS | PX_ADJ><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter);
      break;
    case PX_FWD | PX_LOSS | PX_IMG:
      k_pixels<PX_FWD | PX_LOSS | PX_IMG><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter);
      break;
    case PX_FWD | PX_LOSS:
      k_pixels<PX_FWD | PX_LOSS><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter);
      break;
    case PX_ADJ:
      k_pixels<PX_ADJ><<<grid, PX_THREADS, 0, s>>>(d_jobs, d_items, n_items, d_counter);
      break;
    default:
      throw CudaError("unsupported pixel kernel flags", DRGB_ERR_INVALID);
  }
  count_launch();
}

void launch_loss_finalize(const JobDev* d_jobs, int n_jobs, cudaStream_t s) {
  k_loss_finalize<<<(n_jobs + 63) / 64, 64, 0, s>>>(d_jobs, n_jobs);
  count_launch();
}

}  // namespace drgb
