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
#include "batch.h"

namespace drgb {
// Device memory held by one job (scene, LBVH, views, buffers, optimiser).
int64_t job_device_bytes(const Job& J) {
  int64_t b = 0;
  for (const MeshState& M : J.meshes)
    b += M.vertices.bytes() + M.colors.bytes() + M.tc.bytes() + M.normals.bytes() + M.tangents.bytes() +
         M.transforms.bytes() + M.texture.bytes() + M.rparams.bytes();
  b += J.pos.bytes() + J.orig.bytes() + J.col.bytes() + J.nrm.bytes() + J.tan.bytes() + J.tc.bytes() + J.tri_v.bytes() +
       J.blocks.bytes() + J.meshdev.bytes() + J.block_tr.bytes() + J.vblock.bytes() + J.src_tab.bytes() +
       J.tr_tab.bytes() + J.tr_inv0.bytes();
  b += J.nodes.bytes() + J.nodes4.bytes() + J.tri.bytes() + J.perm.bytes() + J.leaf_of.bytes() + J.leaf_parent.bytes() + J.node_parent.bytes() +
       J.counters.bytes();
  for (int k = 0; k < 2; k++) b += J.sort_keys[k].bytes() + J.sort_vals[k].bytes();
  b += J.sort_hist.bytes() + J.bounds.bytes() + J.edges.bytes() + J.edge_mi.bytes() + J.cams.bytes() + J.ham.bytes();
  b += J.images.bytes() + J.targets.bytes() + J.adj_in.bytes() + J.img_off.bytes() + J.adj.bytes() +
       J.loss_part.bytes() + J.loss_blk.bytes() + J.loss_out.bytes() + J.proj.bytes() + J.pmf.bytes() + J.cdf.bytes() + J.queue.bytes() +
       J.queue_count.bytes() + J.grad.bytes() + J.err.bytes();
  b += J.opt.m.bytes() + J.opt.G.bytes() + J.opt.lr.bytes() + J.opt.iter.bytes() + J.opt.losses.bytes();
  b += J.vis[0].bytes() + J.vis[1].bytes() + J.vis_uv[0].bytes() + J.vis_uv[1].bytes() + J.ra_tiles.bytes() + J.ra_cursor.bytes() + J.ra_state.bytes() +
       J.ra_list.bytes() + J.ra_rec.bytes();
  b += J.sh_grid.bytes() + J.sh_cells.bytes() + J.sh_cursor.bytes() + J.sh_list.bytes() + J.sh_rec.bytes();
  return b;
}

}  // namespace drgb

drgb_renderer* batch_job(drgb_batch* b, int32_t id) {
  auto it = b->jobs.find(id);
  require(it != b->jobs.end(), "unknown batch job id");
  return it->second.get();
}

std::unique_ptr<drgb_renderer> batch_prepare_job(int device, int shading_model, int spp, const drgb_model_params* mp,
                                                 const drgb_scene_desc* scene, const drgb_camera* cams,
                                                 const float* targets, int n_views, const drgb_opt_params* p,
                                                 int deterministic) {
  require(p != nullptr, "null optimiser parameters");
  require(p->n_dmesh_ids <= kBatchMaxDMeshes, "batch jobs have at most 4 differentiable meshes");
  drgb_renderer* r = nullptr;
  int rc = drgb_renderer_create(shading_model, spp, device, &r);
  if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
  std::unique_ptr<drgb_renderer> hold(r);
  if (mp) {
    rc = drgb_renderer_set_model_params(r, mp);
    if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
  }
  if (deterministic) {
    rc = drgb_renderer_set_option(r, DRGB_OPT_DETERMINISTIC, 1);
    if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
  }
  rc = drgb_optimizer_init(r, scene, cams, targets, n_views, p);
  if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
  return hold;
}

int32_t batch_attach(drgb_batch* b, std::unique_ptr<drgb_renderer> r) {
  require(r && r->device == b->device, "job prepared for another device");
  const int32_t id = b->next_id++;
  if (b->bvh_rebuild >= 0) r->bvh_rebuild = b->bvh_rebuild;
  if (b->raster >= 0) {
    const int rc = drgb_renderer_set_option(r.get(), DRGB_OPT_PRIMARY_RASTER, b->raster);
    if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
  }
  b->jobs[id] = std::move(r);
  b->order.push_back(id);
  b->dirty = true;
  return id;
}

void batch_detach(drgb_batch* b, int32_t id) {
  DRGB_CUDA(cudaSetDevice(b->device));
  DRGB_CUDA(cudaStreamSynchronize(b->stream));
  batch_job(b, id);
  b->order.erase(std::find(b->order.begin(), b->order.end(), id));
  std::unique_ptr<drgb_renderer> hold = std::move(b->jobs[id]);
  b->jobs.erase(id);
  hold.reset();
  b->dirty = true;
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
    // set-up runs on the job's own stream; the batch tables are rebuilt
    // (after the batch's stream drains) before the next iteration
    *job_id = batch_attach(b, batch_prepare_job(b->device, shading_model, spp, mp, scene, cams, targets, n_views, p,
                                                b->det));
  });
}

int drgb_batch_remove_job(drgb_batch* b, int32_t id) {
  return guard([&] {
    require(b != nullptr, "null batch");
    batch_detach(b, id);
  });
}

int drgb_batch_size(drgb_batch* b) { return b ? (int)b->order.size() : 0; }

int drgb_batch_set_option(drgb_batch* b, int option, int64_t value) {
  return guard([&] {
    require(b != nullptr, "null batch");
    if (option == DRGB_OPT_USE_GRAPH) {
      b->use_graph = value ? 1 : 0;
    } else if (option == DRGB_OPT_BVH_REBUILD) {
      require(value >= 0 && value <= (1 << 30), "hierarchy rebuild period: 0 (never) or iterations");
      b->bvh_rebuild = (int)value;
      for (auto& kv : b->jobs) kv.second->bvh_rebuild = b->bvh_rebuild;
    } else if (option == DRGB_OPT_PRIMARY_RASTER) {
      require(value >= 0 && value <= 2, "camera and shadow rays: 0, 1 or 2 (see drgb_renderer_set_option)");
      DRGB_CUDA(cudaSetDevice(b->device));
      DRGB_CUDA(cudaStreamSynchronize(b->stream));
      b->raster = (int)value;
      for (auto& kv : b->jobs) {
        const int rc = drgb_renderer_set_option(kv.second.get(), DRGB_OPT_PRIMARY_RASTER, b->raster);
        if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
      }
      b->dirty = true;
    } else if (option == DRGB_OPT_DETERMINISTIC) {
      DRGB_CUDA(cudaSetDevice(b->device));
      DRGB_CUDA(cudaStreamSynchronize(b->stream));
      b->det = value ? 1 : 0;
      for (auto& kv : b->jobs) {
        const int rc = drgb_renderer_set_option(kv.second.get(), DRGB_OPT_DETERMINISTIC, b->det);
        if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
      }
      b->dirty = true;
    } else {
      throw CudaError("unknown batch option", DRGB_ERR_INVALID);
    }
    b->graph_valid = false;
  });
}

// n batched steps: graph replays, or the launches themselves.
static void batch_enqueue_steps(drgb_batch* b, int64_t n_iters) {
  {
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
  }
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
    // steps up to the next job's hierarchy rebuild, which then overlaps the
    // following steps (the job's device pointers stay the same, so the graph
    // stays valid)
    while (n_iters > 0) {
      for (int32_t id : b->order) rebuild_bvh_poll(b->jobs.at(id)->job, b->stream);
      int64_t n = n_iters;
      for (int32_t id : b->order) {
        const drgb_renderer& r = *b->jobs.at(id);
        if (r.bvh_rebuild > 0) n = std::min<int64_t>(n, r.bvh_rebuild - r.job.opt.host_iter % r.bvh_rebuild);
      }
      batch_enqueue_steps(b, n);
      n_iters -= n;
      for (int32_t id : b->order) {
        drgb_renderer& r = *b->jobs.at(id);
        r.job.opt.host_iter += n;
        if (r.bvh_rebuild > 0 && r.job.opt.host_iter % r.bvh_rebuild == 0) rebuild_bvh_begin(r.job, b->stream);
      }
    }
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

int drgb_batch_get_restricted(drgb_batch* b, int32_t id, int mesh_id, float* params) {
  drgb_renderer* r = nullptr;
  int rc = guard([&] {
    require(b != nullptr, "null batch");
    r = batch_job(b, id);
    DRGB_CUDA(cudaSetDevice(b->device));
    DRGB_CUDA(cudaStreamSynchronize(b->stream));
  });
  if (rc != DRGB_OK) return rc;
  return drgb_optimizer_get_restricted(r, mesh_id, params);
}

int drgb_batch_autotune(drgb_batch* b, int trial_iters, int32_t* chosen, float* best_ms) {
  return guard([&] {
    require(b != nullptr && trial_iters >= 1, "bad arguments");
    require(!b->order.empty(), "empty batch", DRGB_ERR_STATE);
    DRGB_CUDA(cudaSetDevice(b->device));
    b->rebuild();
    cudaEvent_t e0, e1;
    DRGB_CUDA(cudaEventCreate(&e0));
    DRGB_CUDA(cudaEventCreate(&e1));
    auto trial = [&] {
      b->enqueue_iteration(false);
      DRGB_CUDA(cudaEventRecord(e0, b->stream));
      for (int i = 0; i < trial_iters; i++) b->enqueue_iteration(false);
      DRGB_CUDA(cudaEventRecord(e1, b->stream));
      DRGB_CUDA(cudaEventSynchronize(e1));
      float ms = 0.0f;
      DRGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms / trial_iters;
    };
    float best = 1e30f;
    for (int which = 0; which < 2; which++) {
      int& knob = which == 0 ? b->px_blocks_per_sm : b->edge_blocks_per_sm;
      int bk = knob;
      for (int k : {2, 4, 8, 16}) {
        knob = k;
        const float ms = trial();
        if (ms < best) {
          best = ms;
          bk = k;
        }
      }
      knob = bk;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->graph_valid = false;
    if (chosen) {
      chosen[0] = b->px_blocks_per_sm;
      chosen[1] = b->edge_blocks_per_sm;
    }
    if (best_ms) *best_ms = best;
  });
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
