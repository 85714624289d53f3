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
  } else if (flags & DRGB_OPT_TFM) {
    if (M.rparams) {
      // translate, rotate, scale -= step (optimizer_simple.cpp:138-160)
      M.rparams[j - M.tr_off] -= v;
    } else {
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
    o.m[k] = opt_mesh(L, M);
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
  launch_restricted_mats(J, s);
}

OptMesh opt_mesh(const DLayout& L, MeshState& M) {
  const bool rt = L.rt_off >= 0;
  return OptMesh{L.base, L.full, L.pos_off, L.color_off, L.tex_off, rt ? L.rt_off : L.tr_off, L.vertices,
                 L.instances, M.vertices.p, M.has_colors ? M.colors.p : nullptr, M.texture.p, M.transforms.p,
                 rt ? M.rparams.p : nullptr};
}

// ---- restricted transforms (TransformR, scene.h:91-116) -------------------
// Row-major 3x4 product with translation, `mul` of drender_autodiff.cpp:22-43.
__device__ void mul34(const float* a, const float* b, float* out) {
  float r[12];
#pragma unroll
  for (int i = 0; i < 3; i++) {
#pragma unroll
    for (int j = 0; j < 3; j++) r[4 * i + j] = a[4 * i + 0] * b[j] + a[4 * i + 1] * b[4 + j] + a[4 * i + 2] * b[8 + j];
    r[4 * i + 3] = a[4 * i + 0] * b[3] + a[4 * i + 1] * b[7] + a[4 * i + 2] * b[11] + a[4 * i + 3];
  }
#pragma unroll
  for (int i = 0; i < 12; i++) out[i] = r[i];
}

// Row q of d(to_mat)/d(params) over the row-major 3x4 entries.  The matrix is
// Rz (Ry (Rx S)) plus the translation column (dmat_dtransforms_jac_f,
// drender_autodiff.cpp:78-95); the derivative by an angle or by the scale
// replaces that factor by its derivative, by a translation it is a unit entry.
// The reference takes these rows from Enzyme's forward mode (:97-107).
__device__ void restricted_jacobian_row(const float* x, int q, float* row) {
  const float sx = sinf(x[3]), cx = cosf(x[3]), sy = sinf(x[4]), cy = cosf(x[4]), sz = sinf(x[5]), cz = cosf(x[5]);
  const float S[12] = {x[6], 0, 0, 0, 0, x[6], 0, 0, 0, 0, x[6], 0};
  const float dS[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  const float Rx[12] = {1, 0, 0, 0, 0, cx, -sx, 0, 0, sx, cx, 0};
  const float Ry[12] = {cy, 0, sy, 0, 0, 1, 0, 0, -sy, 0, cy, 0};
  const float Rz[12] = {cz, -sz, 0, 0, sz, cz, 0, 0, 0, 0, 1, 0};
  const float dRx[12] = {0, 0, 0, 0, 0, -sx, -cx, 0, 0, cx, -sx, 0};
  const float dRy[12] = {-sy, 0, cy, 0, 0, 0, 0, 0, -cy, 0, -sy, 0};
  const float dRz[12] = {-sz, -cz, 0, 0, cz, -sz, 0, 0, 0, 0, 0, 0};
  float a[12], b[12];
  if (q < 3) {
    for (int l = 0; l < 12; l++) row[l] = 0.0f;
    row[4 * q + 3] = 1.0f;
    return;
  }
  mul34(q == 3 ? dRx : Rx, q == 6 ? dS : S, a);
  mul34(q == 4 ? dRy : Ry, a, b);
  mul34(q == 5 ? dRz : Rz, b, row);
}

// grad[rt + 7j + q] += sum_l jac[q][l] * grad[tr12 + 12j + l], l in order
// (drender.h:398-421).
__global__ void k_restricted_grad(float* grad, int64_t rt, int64_t tr12, const float* rparams, int n_inst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 7 * n_inst) return;
  const int j = i / 7, q = i % 7;
  float x[7], row[12];
  for (int k = 0; k < 7; k++) x[k] = rparams[7 * j + k];
  restricted_jacobian_row(x, q, row);
  float acc = grad[rt + i];
  for (int l = 0; l < 12; l++) acc += row[l] * grad[tr12 + 12 * j + l];
  grad[rt + i] = acc;
}

// TransformR::to_mat on the device (column major), LiteMath's product order.
__device__ void mat_mul44(const float* a, const float* b, float* out) {
  float t[16];
  for (int c = 0; c < 4; c++)
    for (int r = 0; r < 4; r++)
      t[4 * c + r] = b[4 * c + 0] * a[r] + b[4 * c + 1] * a[4 + r] + b[4 * c + 2] * a[8 + r] + b[4 * c + 3] * a[12 + r];
  for (int i = 0; i < 16; i++) out[i] = t[i];
}

__global__ void k_restricted_mats(const float* rparams, int n_inst, float* transforms) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_inst) return;
  const float* p = rparams + 7 * j;
  float T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, p[0], p[1], p[2], 1};
  float Rz[16] = {cosf(p[5]), sinf(p[5]), 0, 0, -sinf(p[5]), cosf(p[5]), 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  float Ry[16] = {cosf(p[4]), 0, -sinf(p[4]), 0, 0, 1, 0, 0, sinf(p[4]), 0, cosf(p[4]), 0, 0, 0, 0, 1};
  float Rx[16] = {1, 0, 0, 0, 0, cosf(p[3]), sinf(p[3]), 0, 0, -sinf(p[3]), cosf(p[3]), 0, 0, 0, 0, 1};
  float S[16] = {p[6], 0, 0, 0, 0, p[6], 0, 0, 0, 0, p[6], 0, 0, 0, 0, 1};
  float a[16], b[16];
  mat_mul44(T, Rz, a);
  mat_mul44(a, Ry, b);
  mat_mul44(b, Rx, a);
  mat_mul44(a, S, transforms + 16 * j);
}

void launch_restricted_grad(Job& J, cudaStream_t s) {
  for (const DLayout& L : J.dlay) {
    if (L.rt_off < 0) continue;
    const int n = 7 * L.instances;
    k_restricted_grad<<<(n + 127) / 128, 128, 0, s>>>(J.grad.p, L.base + L.rt_off, L.base + L.tr_off,
                                                      J.meshes[L.mesh_id].rparams.p, L.instances);
    count_launch();
  }
}

void launch_restricted_mats(Job& J, cudaStream_t s) {
  if (!(J.opt.params.flags & DRGB_OPT_TFM)) return;
  for (const DLayout& L : J.dlay) {
    if (L.rt_off < 0) continue;
    MeshState& M = J.meshes[L.mesh_id];
    k_restricted_mats<<<(L.instances + 127) / 128, 128, 0, s>>>(M.rparams.p, L.instances, M.transforms.p);
    count_launch();
  }
}

void launch_opt_record(Job& J, cudaStream_t s) {
  k_opt_record<<<1, 1, 0, s>>>(J.loss_out.p, J.opt.losses.p, (int)J.opt.losses.n, J.opt.iter.p);
  count_launch();
}

}  // namespace drgb
