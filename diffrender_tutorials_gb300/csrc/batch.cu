// Batched optimisation: many independent jobs (meshes, views, resolutions
// and sample counts of uneven size) advanced together, one fused launch
// sequence per iteration for all of them:
//
//   pixel kernel   one persistent launch over the tile work items of every
//                  job (forward + loss + interior adjoint);
//   loss           one block per job;
//   edge pass      segment tables over the (job, view) pairs, one shared
//                  sample queue whose entries carry their job;
//   optimiser      segment tables over the jobs' parameter vectors;
//   flatten/refit  segment tables over the jobs' vertices and triangles.
//
// Each job is set up exactly like a plain optimiser (drgb_optimizer_init on a
// renderer of its own), so the arithmetic per job is the same alone and in
// the mix; only the order of floating-point atomic additions differs.  The
// iteration is captured once in a CUDA graph and replayed.
#include <map>

#include "renderer.h"

namespace drgb {
void launch_b_edges(const JobDev* d_jobs, const Seg* proj_segs, int n_proj, int proj_chunks, const Seg* pmf_segs,
                    int n_pmf, int pmf_chunks, const Seg* pairs, int n_pairs, const Seg* sel_segs, int n_sel,
                    int sel_chunks, int4* queue, int* count, int cap, int shade_grid, cudaStream_t s);
void launch_b_opt(const JobAux* d_aux, int n_jobs, const Seg* d_moment_segs, int n_moment_segs, int moment_chunks,
                  const Seg* d_apply_segs, int n_apply_segs, int apply_chunks, cudaStream_t s);
void launch_b_prepare(const JobAux* d_aux, const Seg* segs[4], const int nsegs[4], const int chunks[4],
                      cudaStream_t s);

// Device memory held by one job (scene, LBVH, views, buffers, optimiser).
int64_t job_device_bytes(const Job& J) {
  int64_t b = 0;
  for (const MeshState& M : J.meshes)
    b += M.vertices.bytes() + M.colors.bytes() + M.tc.bytes() + M.normals.bytes() + M.tangents.bytes() +
         M.transforms.bytes() + M.texture.bytes() + M.indices.bytes();
  b += J.pos.bytes() + J.orig.bytes() + J.col.bytes() + J.nrm.bytes() + J.tc.bytes() + J.tri_v.bytes() +
       J.blocks.bytes() + J.meshdev.bytes() + J.block_tr.bytes() + J.vblock.bytes() + J.src_tab.bytes() +
       J.tr_tab.bytes() + J.tr_inv0.bytes();
  b += J.nodes.bytes() + J.tri.bytes() + J.perm.bytes() + J.leaf_parent.bytes() + J.node_parent.bytes() +
       J.counters.bytes();
  for (int k = 0; k < 2; k++) b += J.sort_keys[k].bytes() + J.sort_vals[k].bytes();
  b += J.sort_hist.bytes() + J.bounds.bytes() + J.edges.bytes() + J.edge_mi.bytes() + J.cams.bytes() + J.ham.bytes();
  b += J.images.bytes() + J.targets.bytes() + J.adj_in.bytes() + J.img_off.bytes() + J.adj.bytes() +
       J.loss_part.bytes() + J.loss_out.bytes() + J.proj.bytes() + J.pmf.bytes() + J.cdf.bytes() + J.queue.bytes() +
       J.queue_count.bytes() + J.grad.bytes() + J.err.bytes();
  b += J.opt.m.bytes() + J.opt.G.bytes() + J.opt.lr.bytes() + J.opt.iter.bytes() + J.opt.losses.bytes();
  return b;
}

}  // namespace drgb

struct drgb_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 1;
  std::map<int32_t, std::unique_ptr<drgb_renderer>> jobs;  // by job id (ordered)
  std::vector<int32_t> order;                              // batch index -> job id
  int32_t next_id = 1;
  bool dirty = true;
  int use_graph = 1;
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;
  int64_t graph_kernels = 0;
  // device tables of the current job set
  DevBuf<JobDev> d_jobs;
  DevBuf<JobAux> d_aux;
  DevBuf<int4> d_items;
  DevBuf<int> d_counter;
  DevBuf<Seg> seg_proj, seg_pmf, seg_pairs, seg_sel, seg_mom, seg_apply, seg_btr, seg_flat, seg_cnt, seg_refit;
  DevBuf<int4> queue;
  DevBuf<int> queue_count;
  int n_items = 0, mode = 0;
  int n_proj = 0, c_proj = 0, n_pmf = 0, c_pmf = 0, n_pairs = 0, n_sel = 0, c_sel = 0;
  int n_mom = 0, c_mom = 0, n_apply = 0, c_apply = 0;
  int n_prep[4] = {0, 0, 0, 0}, c_prep[4] = {0, 0, 0, 0};
  int queue_cap = 0;
  std::vector<JobDev> h_jobs;

  ~drgb_batch() {
    if (graph) cudaGraphExecDestroy(graph);
    if (stream) cudaStreamDestroy(stream);
  }

  // Segment table from (job, sub, count) triples with 256-element chunks.
  static int segs(std::vector<Seg>& out, int& chunks, const std::vector<Seg>& items) {
    out.clear();
    chunks = 0;
    for (Seg s : items) {
      if (s.count <= 0) continue;
      s.begin = chunks;
      chunks += (s.count + 255) / 256;
      out.push_back(s);
    }
    if (out.empty()) out.push_back(Seg{0, 0, 0, 0});
    return (int)out.size();
  }

  void rebuild() {
    if (!dirty) return;
    const int n = (int)order.size();
    h_jobs.assign(n, JobDev{});
    std::vector<JobAux> aux(n);
    std::vector<int4> items;
    std::vector<Seg> proj, pmf, pairs, sel, mom, apply, btr, flat, cnt, refit;
    int modes = -1;
    queue_cap = 0;
    for (int j = 0; j < n; j++) {
      drgb_renderer* r = jobs.at(order[j]).get();
      Job& J = r->job;
      JobDev d = J.dev;
      d.item_base = (int)items.size();
      d.item_count = (int)J.h_pixel_items.size();
      for (int4 it : J.h_pixel_items) items.push_back(make_int4(j, it.y, it.z, it.w));
      h_jobs[j] = d;
      modes = (modes == -1 || modes == J.mode) ? J.mode : 0;
      for (int v = 0; v < J.n_views; v++) {
        proj.push_back(Seg{j, v, 0, J.n_vertices});
        pmf.push_back(Seg{j, v, 0, J.n_edges});
        if (J.n_edges > 0 && d.edge_samples > 0) {
          pairs.push_back(Seg{j, v, 0, 1});
          sel.push_back(Seg{j, v, 0, d.edge_samples});
        }
      }
      queue_cap += J.n_views * std::max(0, d.edge_samples);
      JobAux& A = aux[j];
      A.n_vertices = J.n_vertices;
      A.n_tris = J.n_tris;
      A.n_blocks = J.n_blocks;
      A.vblock = J.vblock.p;
      A.blocks = J.blocks.p;
      A.src = J.src_tab.p;
      A.tr_tab = J.tr_tab.p;
      A.block_tr = J.block_tr.p;
      A.pos = J.pos.p;
      A.orig = J.orig.p;
      A.col = J.col.p;
      A.nrm = J.nrm.p;
      A.tc = J.tc.p;
      A.tri_v = J.tri_v.p;
      A.perm = J.perm.p;
      A.tri = J.tri.p;
      A.nodes = J.nodes.p;
      A.leaf_parent = J.leaf_parent.p;
      A.node_parent = J.node_parent.p;
      A.counters = J.counters.p;
      A.grad = J.grad.p;
      A.grad_total = J.grad_total;
      A.m = J.opt.m.p;
      A.G = J.opt.G.p;
      A.lr = J.opt.lr.p;
      A.iter = J.opt.iter.p;
      A.losses = J.opt.losses.p;
      A.losses_cap = (int)J.opt.losses.n;
      A.loss_out = J.loss_out.p;
      A.alg = J.opt.params.alg;
      A.flags = J.opt.params.flags;
      A.mode = J.mode;
      A.decay_period = J.opt.params.decay_period;
      A.decay_mult = J.opt.params.decay_mult;
      A.n_dmesh = (int)J.dlay.size();
      for (int k = 0; k < A.n_dmesh; k++) {
        const DLayout& L = J.dlay[k];
        MeshState& M = J.meshes[L.mesh_id];
        A.dm[k] = OptMesh{L.base, L.full, L.pos_off, L.color_off, L.tex_off, L.tr_off, L.vertices, L.instances,
                          M.vertices.p, M.has_colors ? M.colors.p : nullptr, M.texture.p, M.transforms.p};
        apply.push_back(Seg{j, k, 0, L.full});
      }
      mom.push_back(Seg{j, 0, 0, J.opt.params.alg >= DRGB_GD_ADAGRAD ? (int)J.grad_total : 0});
      btr.push_back(Seg{j, 0, 0, J.n_blocks});
      flat.push_back(Seg{j, 0, 0, J.n_vertices});
      cnt.push_back(Seg{j, 0, 0, std::max(0, J.n_tris - 1)});
      refit.push_back(Seg{j, 0, 0, J.n_tris});
    }
    mode = modes < 0 ? 0 : modes;
    n_items = (int)items.size();
    std::vector<Seg> t;
    n_proj = segs(t, c_proj, proj);
    seg_proj.upload(t.data(), t.size(), stream);
    n_pmf = segs(t, c_pmf, pmf);
    seg_pmf.upload(t.data(), t.size(), stream);
    n_pairs = (int)pairs.size();
    if (pairs.empty()) pairs.push_back(Seg{0, 0, 0, 0});
    seg_pairs.upload(pairs.data(), pairs.size(), stream);
    n_sel = segs(t, c_sel, sel);
    seg_sel.upload(t.data(), t.size(), stream);
    n_mom = segs(t, c_mom, mom);
    seg_mom.upload(t.data(), t.size(), stream);
    n_apply = segs(t, c_apply, apply);
    seg_apply.upload(t.data(), t.size(), stream);
    n_prep[0] = segs(t, c_prep[0], btr);
    seg_btr.upload(t.data(), t.size(), stream);
    n_prep[1] = segs(t, c_prep[1], flat);
    seg_flat.upload(t.data(), t.size(), stream);
    n_prep[2] = segs(t, c_prep[2], cnt);
    seg_cnt.upload(t.data(), t.size(), stream);
    n_prep[3] = segs(t, c_prep[3], refit);
    seg_refit.upload(t.data(), t.size(), stream);
    d_jobs.upload(h_jobs.data(), h_jobs.size(), stream);
    d_aux.upload(aux.data(), aux.size(), stream);
    d_items.upload(items.data(), items.size(), stream);
    d_counter.alloc(1);
    queue.reserve(std::max(1, queue_cap));
    queue_count.alloc(1);
    DRGB_CUDA(cudaStreamSynchronize(stream));
    dirty = false;
    graph_valid = false;
  }

  void enqueue_iteration() {
    for (int32_t id : order) {
      Job& J = jobs.at(id)->job;
      DRGB_CUDA(cudaMemsetAsync(J.grad.p, 0, sizeof(float) * std::max<int64_t>(1, J.grad_total), stream));
    }
    launch_pixels(d_jobs.p, d_items.p, n_items, d_counter.p, PX_FWD | PX_LOSS | PX_ADJ, sm_count * 8, stream, mode);
    launch_loss_finalize(d_jobs.p, (int)order.size(), stream);
    launch_b_edges(d_jobs.p, seg_proj.p, n_proj, c_proj, seg_pmf.p, n_pmf, c_pmf, seg_pairs.p, n_pairs, seg_sel.p,
                   n_sel, c_sel, queue.p, queue_count.p, (int)queue.n, sm_count * 8, stream);
    launch_b_opt(d_aux.p, (int)order.size(), seg_mom.p, n_mom, c_mom, seg_apply.p, n_apply, c_apply, stream);
    const Seg* sp[4] = {seg_btr.p, seg_flat.p, seg_cnt.p, seg_refit.p};
    launch_b_prepare(d_aux.p, sp, n_prep, c_prep, stream);
  }
};

static drgb_renderer* batch_job(drgb_batch* b, int32_t id) {
  auto it = b->jobs.find(id);
  require(it != b->jobs.end(), "unknown batch job id");
  return it->second.get();
}

extern "C" {

int drgb_batch_create(int device, drgb_batch** out) {
  return guard([&] {
    require(out != nullptr, "null output pointer");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw CudaError("no CUDA device", DRGB_ERR_NO_DEVICE);
    require(device >= 0 && device < n, "device index out of range");
    auto b = std::make_unique<drgb_batch>();
    b->device = device;
    DRGB_CUDA(cudaSetDevice(device));
    DRGB_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    DRGB_CUDA(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, device));
    *out = b.release();
  });
}

int drgb_batch_destroy(drgb_batch* b) {
  if (!b) return DRGB_ERR_INVALID;
  return guard([&] {
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    for (auto& kv : b->jobs) drgb_renderer_destroy(kv.second.release());
    delete b;
  });
}

void* drgb_batch_stream(drgb_batch* b) { return b ? (void*)b->stream : nullptr; }

int drgb_batch_add_job(drgb_batch* b, int shading_model, int spp, const drgb_model_params* mp,
                       const drgb_scene_desc* scene, const drgb_camera* cams, const float* targets, int n_views,
                       const drgb_opt_params* p, int32_t* job_id) {
  return guard([&] {
    require(b && job_id && p, "null argument");
    require(p->n_dmesh_ids <= kBatchMaxDMeshes, "batch jobs have at most 4 differentiable meshes");
    DRGB_CUDA(cudaSetDevice(b->device));
    // the batch's pending work may still read the job tables
    DRGB_CUDA(cudaStreamSynchronize(b->stream));
    drgb_renderer* r = nullptr;
    int rc = drgb_renderer_create(shading_model, spp, b->device, &r);
    if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
    std::unique_ptr<drgb_renderer> hold(r);
    if (mp) {
      rc = drgb_renderer_set_model_params(r, mp);
      if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
    }
    rc = drgb_optimizer_init(r, scene, cams, targets, n_views, p);
    if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
    const int32_t id = b->next_id++;
    b->jobs[id] = std::move(hold);
    b->order.push_back(id);
    b->dirty = true;
    *job_id = id;
  });
}

int drgb_batch_remove_job(drgb_batch* b, int32_t id) {
  return guard([&] {
    require(b != nullptr, "null batch");
    DRGB_CUDA(cudaSetDevice(b->device));
    DRGB_CUDA(cudaStreamSynchronize(b->stream));
    drgb_renderer* r = batch_job(b, id);
    b->order.erase(std::find(b->order.begin(), b->order.end(), id));
    std::unique_ptr<drgb_renderer> hold = std::move(b->jobs[id]);
    b->jobs.erase(id);
    (void)r;
    hold.reset();
    b->dirty = true;
  });
}

int drgb_batch_size(drgb_batch* b) { return b ? (int)b->order.size() : 0; }

int drgb_batch_set_option(drgb_batch* b, int option, int64_t value) {
  return guard([&] {
    require(b != nullptr, "null batch");
    if (option == DRGB_OPT_USE_GRAPH) b->use_graph = value ? 1 : 0;
    else throw CudaError("unknown batch option", DRGB_ERR_INVALID);
    b->graph_valid = false;
  });
}

int drgb_batch_run_async(drgb_batch* b, int64_t n_iters) {
  return guard([&] {
    require(b != nullptr && n_iters >= 0, "bad arguments");
    if (b->order.empty() || n_iters == 0) return;
    DRGB_CUDA(cudaSetDevice(b->device));
    // loss histories must hold the new iterations
    for (int32_t id : b->order) {
      Job& J = b->jobs.at(id)->job;
      if ((int64_t)J.opt.losses.n < J.opt.host_iter + n_iters) {
        size_t cap = std::max<size_t>(1024, J.opt.losses.n);
        while ((int64_t)cap < J.opt.host_iter + n_iters) cap *= 2;
        DevBuf<float> nb;
        nb.alloc(cap);
        DRGB_CUDA(cudaMemcpyAsync(nb.p, J.opt.losses.p, J.opt.losses.bytes(), cudaMemcpyDeviceToDevice, b->stream));
        DRGB_CUDA(cudaStreamSynchronize(b->stream));
        J.opt.losses = std::move(nb);
        b->dirty = true;
      }
    }
    b->rebuild();
    if (b->use_graph) {
      if (!b->graph_valid) {
        if (b->graph) {
          cudaGraphExecDestroy(b->graph);
          b->graph = nullptr;
        }
        int64_t k0 = drgb_kernel_launches();
        cudaGraph_t g;
        DRGB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        try {
          b->enqueue_iteration();
        } catch (...) {
          cudaStreamEndCapture(b->stream, &g);
          throw;
        }
        DRGB_CUDA(cudaStreamEndCapture(b->stream, &g));
        b->graph_kernels = drgb_kernel_launches() - k0;
        DRGB_CUDA(cudaGraphInstantiate(&b->graph, g, 0));
        cudaGraphDestroy(g);
        b->graph_valid = true;
        add_launches(-b->graph_kernels);  // counted per replay below
      }
      for (int64_t i = 0; i < n_iters; i++) DRGB_CUDA(cudaGraphLaunch(b->graph, b->stream));
      add_launches(b->graph_kernels * n_iters);
    } else {
      for (int64_t i = 0; i < n_iters; i++) b->enqueue_iteration();
    }
    for (int32_t id : b->order) b->jobs.at(id)->job.opt.host_iter += n_iters;
  });
}

int drgb_batch_sync(drgb_batch* b) {
  return guard([&] {
    require(b != nullptr, "null batch");
    DRGB_CUDA(cudaSetDevice(b->device));
    DRGB_CUDA(cudaStreamSynchronize(b->stream));
    uint32_t flags = 0;
    for (int32_t id : b->order) {
      uint32_t f = 0;
      DRGB_CUDA(cudaMemcpy(&f, b->jobs.at(id)->job.err.p, sizeof(f), cudaMemcpyDeviceToHost));
      flags |= f;
    }
    if (flags) throw CudaError("kernel error flags " + std::to_string(flags), DRGB_ERR_KERNEL);
  });
}

int drgb_batch_run(drgb_batch* b, int64_t n_iters) {
  const int rc = drgb_batch_run_async(b, n_iters);
  return rc != DRGB_OK ? rc : drgb_batch_sync(b);
}

int drgb_batch_job_losses(drgb_batch* b, int32_t id, int64_t first, int64_t n, float* out, int64_t* iters_done) {
  return guard([&] {
    require(b != nullptr, "null batch");
    drgb_renderer* r = batch_job(b, id);
    DRGB_CUDA(cudaSetDevice(b->device));
    Job& J = r->job;
    if (iters_done) *iters_done = J.opt.host_iter;
    require(first >= 0 && n >= 0 && first + n <= J.opt.host_iter, "loss range beyond the iterations run");
    if (n > 0) {
      DRGB_CUDA(cudaStreamSynchronize(b->stream));
      DRGB_CUDA(cudaMemcpy(out, J.opt.losses.p + first, sizeof(float) * n, cudaMemcpyDeviceToHost));
    }
  });
}

int drgb_batch_get_mesh(drgb_batch* b, int32_t id, int mesh_id, float* vertices, float* colors, float* texture,
                        float* transforms) {
  drgb_renderer* r = nullptr;
  int rc = guard([&] {
    require(b != nullptr, "null batch");
    r = batch_job(b, id);
    DRGB_CUDA(cudaSetDevice(b->device));
    DRGB_CUDA(cudaStreamSynchronize(b->stream));
  });
  if (rc != DRGB_OK) return rc;
  return drgb_optimizer_get_mesh(r, mesh_id, vertices, colors, texture, transforms);
}

int64_t drgb_batch_job_device_bytes(drgb_batch* b, int32_t id) {
  int64_t bytes = -1;
  guard([&] {
    require(b != nullptr, "null batch");
    bytes = job_device_bytes(batch_job(b, id)->job);
  });
  return bytes;
}

}  // extern "C"
