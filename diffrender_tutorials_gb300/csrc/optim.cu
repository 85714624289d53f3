// On-device optimiser: OptSimple::OptStep / OptUpdateScene / StepDecay
// (src/optimizer_simple.cpp:82-236).
//
// The update reproduces the reference exactly, including its "Adam":
//   m <- 0.25 m + 0.75 g;  G <- 2 (0.5 G + 0.5 g^2);  step = m / sqrt(G[i] + 1e-8)
// where G is indexed with the mesh-local index i for every differentiable
// mesh (optimizer_simple.cpp:224), so the moments of all meshes are updated
// before any step is formed.  The learning rate of each gradient segment
// (positions, colours, textures, transforms; GetLR, :61-80) lives in device
// memory and is decayed by a one-thread kernel, so the whole iteration can
// be replayed from a CUDA graph.
#include "engine.h"

namespace drgb {

struct OptDev {
  int n;  // differentiable meshes
  OptMesh m[16];
  int alg, flags, mode;
  int decay_period;
  float decay_mult;
};

__device__ __forceinline__ void opt_moment_body(float* grad, float* m, float* G, int64_t i, int alg) {
  const float g = grad[i];
  if (alg == DRGB_GD_ADAGRAD) {
    G[i] += (g * g);
  } else if (alg == DRGB_GD_RMSPROP) {
    const float alpha = 0.5f;
    G[i] = 2.0f * (G[i] * alpha + (g * g) * (1.0f - alpha));
  } else if (alg == DRGB_GD_ADAM) {
    const float alpha = 0.5f, beta = 0.25f;
    const float mv = m[i] * beta + g * (1.0f - beta);
    m[i] = mv;
    G[i] = 2.0f * (G[i] * alpha + (g * g) * (1.0f - alpha));
    grad[i] = mv;
  }
}

__global__ void k_opt_moments(float* grad, float* m, float* G, int64_t n, int alg) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  opt_moment_body(grad, m, G, i, alg);
}

// Step of element j of differentiable mesh k: scale, then subtract from the
// scene parameter it belongs to (OptStep + OptUpdateScene).
__device__ __forceinline__ void opt_apply_body(float* grad, const float* G, const float* lr, const OptMesh& M, int k,
                                               int j, int alg, int flags, int mode) {
  float v = grad[M.base + j];
  if (alg >= DRGB_GD_ADAGRAD) v = v / (sqrtf(G[j] + 1e-8f));
  // segment of j: positions [0, color|tex|tr), colours, texture, transforms
  int seg;
  if (j >= M.tr_off) seg = 3;
  else if (M.tex_off >= 0 && j >= M.tex_off) seg = 2;
  else if (M.color_off >= 0 && j >= M.color_off) seg = 1;
  else seg = 0;
  v *= lr[4 * k + seg];
  grad[M.base + j] = v;
  if (seg == 0) {
    if (flags & DRGB_OPT_POS) M.vertices[j - M.pos_off] -= v;
  } else if (seg == 1) {
    if ((flags & DRGB_OPT_COL) && M.colors) M.colors[j - M.color_off] -= v;
  } else if (seg == 2) {
    if ((flags & DRGB_OPT_TEX) && mode != SILHOUETTE && mode != VERTEX_COLOR && M.texture)
      M.texture[j - M.tex_off] -= v;
  } else {
    if (flags & DRGB_OPT_TFM) {
      const int l = j - M.tr_off, inst = l / 12, r = (l % 12) / 4, c = l % 4;
      M.transforms[16 * inst + 4 * c + r] -= v;
    }
  }
}

__global__ void k_opt_apply(float* grad, const float* G, const float* lr, OptDev o) {
  const int k = blockIdx.y;
  if (k >= o.n) return;
  const OptMesh& M = o.m[k];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M.full) return;
  opt_apply_body(grad, G, lr, M, k, j, o.alg, o.flags, o.mode);
}

// ---- batched forms: one launch over the parameters of many jobs ----------
__global__ void k_b_opt_moments(const JobAux* aux, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int64_t i = (int64_t)(blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (i >= sg.count) return;
  const JobAux& A = aux[sg.job];
  if (A.alg >= DRGB_GD_ADAGRAD) opt_moment_body(A.grad, A.m, A.G, i, A.alg);
}

__global__ void k_b_opt_apply(const JobAux* aux, const Seg* segs, int nseg) {
  const Seg sg = segs[find_seg(segs, nseg, blockIdx.x)];
  const int j = (blockIdx.x - sg.begin) * blockDim.x + threadIdx.x;
  if (j >= sg.count) return;
  const JobAux& A = aux[sg.job];
  opt_apply_body(A.grad, A.G, A.lr, A.dm[sg.sub], sg.sub, j, A.alg, A.flags, A.mode);
}

// Per job: losses[iter] = loss, StepDecay(iter), iter++.
__global__ void k_b_opt_tail(const JobAux* aux, int n_jobs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_jobs) return;
  const JobAux& A = aux[j];
  const int it = *A.iter;
  if (it >= 0 && it < A.losses_cap) A.losses[it] = *A.loss_out;
  if (it > 0 && it % max(1, A.decay_period) == 0)
    for (int i = 0; i < 4 * A.n_dmesh; i++) A.lr[i] *= A.decay_mult;
  *A.iter = it + 1;
}

void launch_b_opt(const JobAux* d_aux, int n_jobs, const Seg* d_moment_segs, int n_moment_segs, int moment_chunks,
                  const Seg* d_apply_segs, int n_apply_segs, int apply_chunks, cudaStream_t s) {
  if (moment_chunks > 0) k_b_opt_moments<<<moment_chunks, 256, 0, s>>>(d_aux, d_moment_segs, n_moment_segs);
  if (apply_chunks > 0) k_b_opt_apply<<<apply_chunks, 256, 0, s>>>(d_aux, d_apply_segs, n_apply_segs);
  k_b_opt_tail<<<(n_jobs + 127) / 128, 128, 0, s>>>(d_aux, n_jobs);
  count_launch(3);
}

// StepDecay(iter) then iter++ (optimizer_simple.cpp:82-90, 293-301).
__global__ void k_opt_decay(float* lr, int n_lr, int* iter, int period, float mult) {
  const int it = *iter;
  if (it > 0 && it % period == 0)
    for (int i = 0; i < n_lr; i++) lr[i] *= mult;
  *iter = it + 1;
}

// Loss history: losses[iter] = loss of this iteration.
__global__ void k_opt_record(const float* loss, float* hist, int cap, const int* iter) {
  const int it = *iter;
  if (it >= 0 && it < cap) hist[it] = *loss;
}

void launch_opt_step(Job& J, cudaStream_t s) {
  OptDev o{};
  o.n = (int)J.dlay.size();
  o.alg = J.opt.params.alg;
  o.flags = J.opt.params.flags;
  o.mode = J.mode;
  o.decay_period = J.opt.params.decay_period;
  o.decay_mult = J.opt.params.decay_mult;
  int max_full = 0;
  for (int k = 0; k < o.n; k++) {
    const DLayout& L = J.dlay[k];
    MeshState& M = J.meshes[L.mesh_id];
    o.m[k] = OptMesh{L.base, L.full, L.pos_off, L.color_off, L.tex_off, L.tr_off, L.vertices, L.instances,
                     M.vertices.p, M.has_colors ? M.colors.p : nullptr, M.texture.p, M.transforms.p};
    max_full = std::max(max_full, L.full);
  }
  if (J.opt.params.alg >= DRGB_GD_ADAGRAD) {
    k_opt_moments<<<(unsigned)((J.grad_total + 255) / 256), 256, 0, s>>>(J.grad.p, J.opt.m.p, J.opt.G.p,
                                                                         J.grad_total, J.opt.params.alg);
    count_launch();
  }
  const dim3 g((max_full + 255) / 256, o.n);
  k_opt_apply<<<g, 256, 0, s>>>(J.grad.p, J.opt.G.p, J.opt.lr.p, o);
  k_opt_decay<<<1, 1, 0, s>>>(J.opt.lr.p, 4 * o.n, J.opt.iter.p, std::max(1, o.decay_period), o.decay_mult);
  count_launch(2);
}

void launch_opt_record(Job& J, cudaStream_t s) {
  k_opt_record<<<1, 1, 0, s>>>(J.loss_out.p, J.opt.losses.p, (int)J.opt.losses.n, J.opt.iter.p);
  count_launch();
}

}  // namespace drgb
