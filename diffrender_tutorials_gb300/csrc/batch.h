// The batch object behind drgb_batch_* and the serving loop: a set of
// independent optimisation jobs advanced by one fused launch sequence per
// iteration (see batch.cu).
#pragma once
#include <map>

#include "renderer.h"

namespace drgb {
void launch_b_edges(const JobDev* d_jobs, const Seg* proj_segs, int n_proj, int proj_chunks, const Seg* pmf_segs,
                    int n_pmf, int pmf_chunks, const Seg* pairs, int n_pairs, const Seg* sel_segs, int n_sel,
                    int sel_chunks, int4* queue, int* count, int cap, int shade_grid, cudaStream_t s, bool det,
                    const QueueSort* qs);
void launch_b_opt(const JobAux* d_aux, int n_jobs, const Seg* d_moment_segs, int n_moment_segs, int moment_chunks,
                  const Seg* d_apply_segs, int n_apply_segs, int apply_chunks, cudaStream_t s);
void launch_b_prepare(const JobAux* d_aux, const Seg* segs[4], const int nsegs[4], const int chunks[4],
                      cudaStream_t s);

int64_t job_device_bytes(const Job& J);
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
  int det = 0;      // deterministic gradient reduction for every job added
  int bvh_rebuild = -1;  // hierarchy rebuild period for every job (-1: the jobs' own)
  int raster = -1;       // DRGB_OPT_PRIMARY_RASTER for every job (-1: the jobs' own)
  bool det_any = false;  // some job of the current set reduces deterministically
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
  DevBuf<uint32_t> qkey[2], qhist;  // shading order of the queue, sorted by (job, view, edge)
  DevBuf<int> qidx[2], qn;
  int qbits = 1;
  int n_items = 0;
  struct ModeGroup {
    int mode, begin, count;  // contiguous pixel items of one shading model
  };
  std::vector<ModeGroup> mode_groups;
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
    // the previous iteration may still read the tables replaced below
    DRGB_CUDA(cudaStreamSynchronize(stream));
    const int n = (int)order.size();
    h_jobs.assign(n, JobDev{});
    std::vector<JobAux> aux(n);
    std::vector<int4> items;
    std::vector<Seg> proj, pmf, pairs, sel, mom, apply, btr, flat, cnt, refit;
    // jobs grouped by shading model: each group's pixel items run in the
    // kernel specialised for that model (item_base is relative to the group)
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return jobs.at(a)->job.mode < jobs.at(b)->job.mode; });
    mode_groups.clear();
    queue_cap = 0;
    uint64_t key_base = 0;
    for (int j = 0; j < n; j++) {
      drgb_renderer* r = jobs.at(order[j]).get();
      Job& J = r->job;
      JobDev d = J.dev;
      d.top_n = 0;  // batched kernels stage no job's top levels
      // a job's raster buffers and light cells (its own; see enqueue_iteration)
      d.edge_key_base = (uint32_t)key_base;
      key_base += (uint64_t)J.n_views * (uint64_t)std::max(0, J.n_edges);
      if (mode_groups.empty() || mode_groups.back().mode != J.mode)
        mode_groups.push_back(ModeGroup{J.mode, (int)items.size(), 0});
      d.item_base = (int)items.size() - mode_groups.back().begin;
      d.item_count = (int)J.h_pixel_items.size();
      for (int4 it : J.h_pixel_items) items.push_back(make_int4(j, it.y, it.z, it.w));
      mode_groups.back().count += d.item_count;
      h_jobs[j] = d;
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
      A.tan = J.tan.p;
      A.tc = J.tc.p;
      A.tri_v = J.tri_v.p;
      A.perm = J.perm.p;
      A.leaf_of = J.leaf_of.p;
      A.tri = J.tri.p;
      A.nodes = J.nodes.p;
      A.nodes4 = J.nodes4.p;
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
        A.dm[k] = opt_mesh(L, M);
        apply.push_back(Seg{j, k, 0, L.full});
      }
      mom.push_back(Seg{j, 0, 0, J.opt.params.alg >= DRGB_GD_ADAGRAD ? (int)J.grad_total : 0});
      btr.push_back(Seg{j, 0, 0, J.n_blocks});
      flat.push_back(Seg{j, 0, 0, J.n_vertices});
      cnt.push_back(Seg{j, 0, 0, std::max(0, J.n_tris - 1)});
      refit.push_back(Seg{j, 0, 0, J.n_tris});
    }
    n_items = (int)items.size();
    det_any = false;
    for (int32_t id : order) det_any = det_any || jobs.at(id)->job.det;
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
    d_counter.alloc(std::max<size_t>(1, mode_groups.size()));
    queue.reserve(std::max(1, queue_cap));
    queue_count.alloc(2);  // [0] queue entries, [1] shading counter
    for (int b = 0; b < 2; b++) {
      qkey[b].reserve(queue.n);
      qidx[b].reserve(queue.n);
    }
    qhist.reserve(scan_scratch(256 * (size_t)kSortGrid));
    qn.reserve(1);
    qbits = 1;
    while (qbits < 32 && (1ull << qbits) < std::max<uint64_t>(1, key_base)) qbits++;
    DRGB_CUDA(cudaStreamSynchronize(stream));
    dirty = false;
    graph_valid = false;
  }

  int px_blocks_per_sm = 8, edge_blocks_per_sm = 8;  // shared persistent grids (autotuned)

  // update = false: the gradient passes only (autotuning; state unchanged)
  void enqueue_iteration(bool update = true) {
    const QueueSort qsort{{qkey[0].p, qkey[1].p}, {qidx[0].p, qidx[1].p}, qhist.p, qn.p, qbits};
    for (int32_t id : order) {
      Job& J = jobs.at(id)->job;
      DRGB_CUDA(cudaMemsetAsync(J.grad.p, 0, J.grad_bytes(), stream));
    }
    for (int32_t id : order) {
      Job& J = jobs.at(id)->job;
      if (J.det && J.rec_key.p) launch_det_clear(J, stream);
    }
    // each job's raster pass and light cells (jobs without them trace)
    int vis = 0;
    for (size_t j = 0; j < order.size(); j++)
      vis |= jobs.at(order[j])->raster_pass(PX_FWD | PX_ADJ, d_jobs.p + j, stream);
    for (size_t g = 0; g < mode_groups.size(); g++)
      launch_pixels(d_jobs.p, d_items.p + mode_groups[g].begin, mode_groups[g].count, d_counter.p + g,
                    PX_FWD | PX_LOSS | PX_ADJ | vis, sm_count * px_blocks_per_sm, stream, mode_groups[g].mode,
                    det_any);
    launch_loss_finalize(d_jobs.p, (int)order.size(), stream);
    launch_b_edges(d_jobs.p, seg_proj.p, n_proj, c_proj, seg_pmf.p, n_pmf, c_pmf, seg_pairs.p, n_pairs, seg_sel.p,
                   n_sel, c_sel, queue.p, queue_count.p, (int)queue.n, sm_count * edge_blocks_per_sm, stream,
                   det_any, &qsort);
    for (int32_t id : order) {
      Job& J = jobs.at(id)->job;
      if (J.det && J.rec_key.p) launch_det_reduce(J, sm_count, stream);
      launch_restricted_grad(J, stream);
    }
    if (!update) return;
    launch_b_opt(d_aux.p, (int)order.size(), seg_mom.p, n_mom, c_mom, seg_apply.p, n_apply, c_apply, stream);
    for (int32_t id : order) launch_restricted_mats(jobs.at(id)->job, stream);
    const Seg* sp[4] = {seg_btr.p, seg_flat.p, seg_cnt.p, seg_refit.p};
    launch_b_prepare(d_aux.p, sp, n_prep, c_prep, stream);
  }
};


// A job prepared outside the batch (renderer + optimiser state on the job's
// own stream), so that its set-up can overlap a running batch iteration.
std::unique_ptr<drgb_renderer> batch_prepare_job(int device, int shading_model, int spp, const drgb_model_params* mp,
                                                 const drgb_scene_desc* scene, const drgb_camera* cams,
                                                 const float* targets, int n_views, const drgb_opt_params* p,
                                                 int deterministic);
// Adds a prepared job; the device tables are rebuilt before the next iteration.
int32_t batch_attach(drgb_batch* b, std::unique_ptr<drgb_renderer> r);
// Removes a job and frees its device memory (waits for the batch's stream).
void batch_detach(drgb_batch* b, int32_t id);
drgb_renderer* batch_job(drgb_batch* b, int32_t id);
