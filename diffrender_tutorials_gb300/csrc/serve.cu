// Serving loop: mesh-optimisation jobs submitted at any time, admitted by a
// device-memory budget and a slot count, advanced together by continuous
// batching on one GPU.
//
// A job is one IOptimizer::Init + Run(n_steps) (src/optimizer.h:52-61,
// src/optimizer_simple.cpp:25-309).  Per step of the server:
//
//   1. the batched iteration of the resident jobs is enqueued (a CUDA graph
//      replay on the batch's stream, bracketed by events);
//   2. while it runs, queued jobs are admitted in arrival order as long as a
//      slot is free and their estimated device bytes fit the budget: each is
//      set up (upload, flatten, LBVH build, optimiser state) on its own
//      stream, overlapping the batched iteration;
//   3. after the iteration, jobs that reached their step count are retired:
//      final meshes and loss history go to host memory, device memory is
//      freed; the new jobs join the batch for the next step.
//
// Host inputs are copied at submission, so a client can free them at once.
// Times are on one steady clock that starts with the server.
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "batch.h"

namespace {

using Clock = std::chrono::steady_clock;

// Host copy of a scene description and its arrays.
struct HostScene {
  std::vector<std::vector<float>> v, col, tc, nrm, tan, tr, tex, rt;
  std::vector<std::vector<uint32_t>> idx;
  std::vector<drgb_mesh_desc> meshes;
  drgb_scene_desc desc{};

  template <class T>
  static std::vector<T> take(const T* p, size_t n) {
    return p ? std::vector<T>(p, p + n) : std::vector<T>();
  }

  explicit HostScene(const drgb_scene_desc& s) {
    const int n = s.n_meshes;
    v.resize(n); col.resize(n); tc.resize(n); nrm.resize(n); tan.resize(n); tr.resize(n); tex.resize(n);
    rt.resize(n);
    idx.resize(n);
    meshes.resize(n);
    for (int i = 0; i < n; i++) {
      const drgb_mesh_desc& m = s.meshes[i];
      const size_t nv = (size_t)std::max(0, m.n_vertices);
      v[i] = take(m.vertices, 3 * nv);
      col[i] = take(m.colors, 3 * nv);
      tc[i] = take(m.tc, 2 * nv);
      nrm[i] = take(m.normals, 3 * nv);
      tan[i] = take(m.tangents, 3 * nv);
      idx[i] = take(m.indices, (size_t)std::max(0, m.n_indices));
      tr[i] = take(m.transforms, 16 * (size_t)std::max(0, m.n_instances));
      tex[i] = take(m.texture, (size_t)std::max(0, m.tex_w) * std::max(0, m.tex_h) * std::max(0, m.tex_channels));
      rt[i] = take(m.restricted, 7 * (size_t)std::max(1, m.n_instances));
      drgb_mesh_desc d = m;
      d.vertices = v[i].empty() ? nullptr : v[i].data();
      d.colors = col[i].empty() ? nullptr : col[i].data();
      d.tc = tc[i].empty() ? nullptr : tc[i].data();
      d.normals = nrm[i].empty() ? nullptr : nrm[i].data();
      d.tangents = tan[i].empty() ? nullptr : tan[i].data();
      d.indices = idx[i].empty() ? nullptr : idx[i].data();
      d.transforms = tr[i].empty() ? nullptr : tr[i].data();
      d.texture = tex[i].empty() ? nullptr : tex[i].data();
      d.restricted = rt[i].empty() ? nullptr : rt[i].data();
      meshes[i] = d;
    }
    desc.n_meshes = n;
    desc.meshes = meshes.data();
  }
};

struct Ticket {
  // request (dropped once admitted)
  int mode = 0, spp = 0;
  drgb_model_params mp{};
  bool has_mp = false;
  std::unique_ptr<HostScene> scene;
  std::vector<drgb_camera> cams;
  std::vector<float> targets;
  drgb_opt_params params{};
  // state
  drgb_job_info info{};
  int32_t batch_id = 0;
  // results
  std::vector<float> losses;
  std::vector<std::vector<float>> out_v, out_col, out_tex, out_tr, out_rt;
};

int64_t estimate_bytes(const drgb_scene_desc& s, const drgb_camera* cams, int n_views, int spp, int mode) {
  int64_t V = 0, T = 0, VF = 0, TF = 0, tex = 0, inst = 0;
  for (int i = 0; i < s.n_meshes; i++) {
    const drgb_mesh_desc& m = s.meshes[i];
    const int64_t ni = std::max(1, m.n_instances);
    V += m.n_vertices;
    T += m.n_indices / 3;
    VF += (int64_t)m.n_vertices * ni;
    TF += (int64_t)(m.n_indices / 3) * ni;
    tex += (int64_t)std::max(0, m.tex_w) * std::max(0, m.tex_h) * std::max(0, m.tex_channels);
    inst += ni;
  }
  int64_t px = 0;
  for (int k = 0; k < n_views; k++) px += (int64_t)cams[k].width * (int64_t)cams[k].height;
  const int64_t nv = std::max(1, n_views);
  int64_t b = 0;
  b += V * 56 + T * 12 + tex * 4 + inst * 128;  // mesh arrays, transforms and inverses
  b += VF * (72 + 4 + 16 * nv);                 // flattened vertices, vertex blocks, projections
  if (mode == PATH_TEST) b += VF * 16;          // flattened tangents
  b += TF * (16 + 272);                         // triangle ids, LBVH nodes (binary, 4-wide builds), leaves, sort buffers
  b += TF * (72 + 24 * nv);                     // edges (at most 3 per triangle), pmf/CDF per view
  b += px * (12 + 16 + 8 + 16 + 8);             // targets, adjoint, loss partials, edge queue, random table
  b += (V * 6 + tex + inst * 12) * 4 * 3;       // gradient, first and second moments
  b += 64 << 10;                                // tables, counters, loss history
  // raster pass: a hit record per forward and adjoint sample (with u, v
  // beside it for the point-light model), per (view,
  // triangle) a footprint and room for 32 tile-list entries, tile offsets;
  // the light-space cells of the point-light models (64 entries per triangle)
  const int64_t S = (int64_t)std::max(1, (int)std::sqrt((float)std::max(1, spp))) *
                    std::max(1, (int)std::sqrt((float)std::max(1, spp)));
  // (the renderer's size rule)
  if (!raster_pays(px * S, nv, TF)) return b;
  b += px * S * (vis_points(mode) ? 48 : 32) + TF * nv * (64 + 128) + (int64_t)(1 << 16) * 4 + px * 8 + 64;
  if (mode == LAMBERT_POINT_VCOLOR || mode == PATH_DIFFUSE) {
    const int64_t G = light_grid_size((int)std::min<int64_t>(TF, 1 << 30));
    b += G * G * 8 + 16 + TF * (64 + 256) + (int64_t)(1 << 16) * 4 + 64;
  }
  return b;
}

}  // namespace

struct drgb_server {
  drgb_server_config cfg{};
  drgb_batch* batch = nullptr;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int32_t> queue;
  std::unordered_map<int32_t, std::unique_ptr<Ticket>> tickets;
  std::unordered_map<int32_t, int32_t> by_batch_id;  // batch job id -> ticket
  int32_t next_ticket = 1;
  int64_t bytes_in_use = 0, bytes_peak = 0;
  int64_t batch_steps = 0, job_iterations = 0;
  double busy = 0.0;
  int32_t n_done = 0, n_failed = 0;
  std::vector<float> step_ms;
  std::vector<int32_t> step_jobs;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::thread worker;
  bool stop = false;
  bool stepping = false;  // a step is in progress (worker or caller)

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  // Called with mu held.
  bool has_work() const { return !queue.empty() || (batch && drgb_batch_size(batch) > 0); }

  void fail_job(Ticket& t, int code) {
    t.info.state = DRGB_JOB_FAILED;
    t.info.error = code;
    t.info.t_done = now();
    n_failed++;
  }

  // Admits queued jobs that fit (arrival order, no overtaking).  Runs while
  // the batch's iteration is in flight; touches the batch only through
  // batch_prepare_job (the job's own stream).
  std::vector<std::pair<int32_t, std::unique_ptr<drgb_renderer>>> admit() {
    std::vector<std::pair<int32_t, std::unique_ptr<drgb_renderer>>> ready;
    for (;;) {
      int32_t id;
      Ticket* t;
      {
        std::lock_guard<std::mutex> lk(mu);
        if (queue.empty()) break;
        id = queue.front();
        t = tickets.at(id).get();
        const int resident = drgb_batch_size(batch) + (int)ready.size();
        if (cfg.max_jobs > 0 && resident >= cfg.max_jobs) break;
        if (bytes_in_use + t->info.device_bytes > cfg.hbm_budget_bytes) break;
        queue.pop_front();
        bytes_in_use += t->info.device_bytes;  // reserved at the estimate until measured
      }
      std::unique_ptr<drgb_renderer> r;
      int code = guard([&] {
        r = batch_prepare_job(cfg.device, t->mode, t->spp, t->has_mp ? &t->mp : nullptr, &t->scene->desc,
                              t->cams.data(), t->targets.data(), (int)t->cams.size(), &t->params,
                              cfg.deterministic);
      });
      std::lock_guard<std::mutex> lk(mu);
      bytes_in_use -= t->info.device_bytes;
      if (code != DRGB_OK) {
        fail_job(*t, code);
        cv_done.notify_all();
        continue;
      }
      t->info.device_bytes = job_device_bytes(r->job);
      bytes_in_use += t->info.device_bytes;
      bytes_peak = std::max(bytes_peak, bytes_in_use);
      ready.emplace_back(id, std::move(r));
    }
    return ready;
  }

  // Copies a finished job's results to host memory and frees it.
  void retire(int32_t tid) {
    Ticket& t = *tickets.at(tid);
    drgb_renderer* r = batch_job(batch, t.batch_id);
    Job& J = r->job;
    const int64_t n = J.opt.host_iter;
    t.losses.resize((size_t)n);
    if (n) DRGB_CUDA(cudaMemcpy(t.losses.data(), J.opt.losses.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    const int nm = (int)J.meshes.size();
    t.out_v.resize(nm); t.out_col.resize(nm); t.out_tex.resize(nm); t.out_tr.resize(nm); t.out_rt.resize(nm);
    for (int m = 0; m < nm; m++) {
      const MeshState& M = J.meshes[m];
      t.out_v[m].resize(3 * (size_t)M.nv);
      if (M.has_colors) t.out_col[m].resize(3 * (size_t)M.nv);
      t.out_tex[m].resize(M.texture.n);
      t.out_tr[m].resize(M.transforms.n);
      const int rc = drgb_optimizer_get_mesh(r, m, t.out_v[m].data(), M.has_colors ? t.out_col[m].data() : nullptr,
                                             t.out_tex[m].empty() ? nullptr : t.out_tex[m].data(),
                                             t.out_tr[m].empty() ? nullptr : t.out_tr[m].data());
      if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
      if (M.restricted) {
        t.out_rt[m].resize(M.rparams.n);
        const int rc2 = drgb_optimizer_get_restricted(r, m, t.out_rt[m].data());
        if (rc2 != DRGB_OK) throw CudaError(t_err_message(), rc2);
      }
    }
    batch_detach(batch, t.batch_id);
    std::lock_guard<std::mutex> lk(mu);
    by_batch_id.erase(t.batch_id);
    t.batch_id = 0;
    bytes_in_use -= t.info.device_bytes;
    t.info.state = DRGB_JOB_DONE;
    t.info.final_loss = t.losses.empty() ? 0.0f : t.losses.back();
    t.info.t_done = now();
    n_done++;
  }

  void step() {
    const int running = drgb_batch_size(batch);
    bool launched = false;
    if (running > 0) {
      DRGB_CUDA(cudaEventRecord(ev0, drgb_batch_stream_t(batch)));
      const int rc = drgb_batch_run_async(batch, 1);
      if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
      DRGB_CUDA(cudaEventRecord(ev1, drgb_batch_stream_t(batch)));
      launched = true;
    }
    auto ready = admit();  // overlaps the iteration in flight
    if (launched) {
      const int rc = drgb_batch_sync(batch);
      if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
      float ms = 0.0f;
      DRGB_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
      std::vector<int32_t> finished;
      {
        std::lock_guard<std::mutex> lk(mu);
        step_ms.push_back(ms);
        step_jobs.push_back(running);
        busy += ms * 1e-3;
        batch_steps++;
        job_iterations += running;
        for (int32_t bid : batch->order) {
          Ticket& t = *tickets.at(by_batch_id.at(bid));
          t.info.steps_done++;
          if (t.info.steps_done >= t.info.steps) finished.push_back(by_batch_id.at(bid));
        }
      }
      for (int32_t tid : finished) retire(tid);
      if (!finished.empty()) cv_done.notify_all();
    }
    for (auto& pr : ready) {
      const int32_t bid = batch_attach(batch, std::move(pr.second));
      std::lock_guard<std::mutex> lk(mu);
      Ticket& t = *tickets.at(pr.first);
      t.batch_id = bid;
      by_batch_id[bid] = pr.first;
      t.info.state = DRGB_JOB_RUNNING;
      t.info.t_admit = now();
      // the request copies are no longer needed
      t.scene.reset();
      std::vector<float>().swap(t.targets);
    }
  }

  // A failed step fails every resident job and empties the batch.
  void fail_resident(int code) {
    std::vector<int32_t> ids;
    {
      std::lock_guard<std::mutex> lk(mu);
      for (auto& kv : by_batch_id) ids.push_back(kv.first);
    }
    for (int32_t bid : ids) {
      guard([&] { batch_detach(batch, bid); });
      std::lock_guard<std::mutex> lk(mu);
      Ticket& t = *tickets.at(by_batch_id.at(bid));
      bytes_in_use -= t.info.device_bytes;
      t.batch_id = 0;
      fail_job(t, code);
      by_batch_id.erase(bid);
    }
    cv_done.notify_all();
  }

  int step_guarded() {
    {
      std::lock_guard<std::mutex> lk(mu);
      stepping = true;
    }
    const int code = guard([&] { step(); });
    if (code != DRGB_OK) {
      const std::string msg = t_err_message();
      fail_resident(code);
      drgb_set_last_error(msg);
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      stepping = false;
    }
    cv_done.notify_all();
    return code;
  }

  void worker_loop() {
    cudaSetDevice(cfg.device);
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || has_work(); });
        if (stop) return;
      }
      step_guarded();
    }
  }

  static cudaStream_t drgb_batch_stream_t(drgb_batch* b) { return (cudaStream_t)drgb_batch_stream(b); }
};

static Ticket& find_ticket(drgb_server* s, int32_t id) {
  auto it = s->tickets.find(id);
  require(it != s->tickets.end(), "unknown ticket");
  return *it->second;
}

extern "C" {

int64_t drgb_estimate_job_bytes(int shading_model, int spp, const drgb_scene_desc* scene, const drgb_camera* cams,
                                int n_views) {
  if (!scene || !cams || n_views <= 0) return -1;
  return estimate_bytes(*scene, cams, n_views, spp, shading_model);
}

int drgb_server_create(const drgb_server_config* cfg, drgb_server** out) {
  return guard([&] {
    require(cfg && out, "null argument");
    *out = nullptr;
    require(cfg->hbm_budget_bytes > 0, "memory budget must be positive");
    auto s = std::make_unique<drgb_server>();
    s->cfg = *cfg;
    s->t0 = Clock::now();
    int rc = drgb_batch_create(cfg->device, &s->batch);
    if (rc != DRGB_OK) throw CudaError(t_err_message(), rc);
    DRGB_CUDA(cudaEventCreate(&s->ev0));
    DRGB_CUDA(cudaEventCreate(&s->ev1));
    if (cfg->start_worker) s->worker = std::thread([p = s.get()] { p->worker_loop(); });
    *out = s.release();
  });
}

int drgb_server_destroy(drgb_server* s) {
  if (!s) return DRGB_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  const int rc = drgb_batch_destroy(s->batch);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  delete s;
  return rc;
}

int drgb_server_submit(drgb_server* s, int shading_model, int spp, const drgb_model_params* mp,
                       const drgb_scene_desc* scene, const drgb_camera* cams, const float* targets, int n_views,
                       const drgb_opt_params* p, int64_t n_steps, int32_t* ticket) {
  return guard([&] {
    require(s && scene && cams && targets && p && ticket, "null argument");
    require(n_views > 0 && n_steps > 0, "need at least one view and one step");
    require(scene->n_meshes > 0 && scene->meshes, "empty scene");
    require(p->n_dmesh_ids >= 1 && p->n_dmesh_ids <= kBatchMaxDMeshes, "need 1..4 differentiable meshes");
    for (int k = 1; k < n_views; k++)
      require((int)cams[k].width == (int)cams[0].width && (int)cams[k].height == (int)cams[0].height,
              "gradient calls need all views of the same size");
    auto t = std::make_unique<Ticket>();
    t->mode = shading_model;
    t->spp = spp;
    if (mp) {
      t->mp = *mp;
      t->has_mp = true;
    }
    t->scene = std::make_unique<HostScene>(*scene);
    t->cams.assign(cams, cams + n_views);
    const size_t npix = (size_t)n_views * (size_t)cams[0].width * (size_t)cams[0].height;
    t->targets.assign(targets, targets + 3 * npix);
    t->params = *p;
    t->info.state = DRGB_JOB_QUEUED;
    t->info.steps = n_steps;
    t->info.t_admit = t->info.t_done = -1.0;
    t->info.device_bytes = estimate_bytes(*scene, cams, n_views, spp, shading_model);
    if (t->info.device_bytes > s->cfg.hbm_budget_bytes)
      throw CudaError("job needs more device memory than the whole budget", DRGB_ERR_OOM);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      t->info.t_submit = s->now();
      const int32_t id = s->next_ticket++;
      s->queue.push_back(id);
      s->tickets[id] = std::move(t);
      *ticket = id;
    }
    s->cv_work.notify_all();
  });
}

int drgb_server_step(drgb_server* s, int32_t* n_running) {
  if (!s) return DRGB_ERR_INVALID;
  if (s->cfg.start_worker) {
    drgb_set_last_error("the server has a worker thread; drgb_server_step is for servers without one");
    return DRGB_ERR_STATE;
  }
  const int rc = s->step_guarded();
  if (n_running) *n_running = drgb_batch_size(s->batch);
  return rc;
}

int drgb_server_wait(drgb_server* s, int32_t ticket, double timeout_s) {
  return guard([&] {
    require(s != nullptr, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&] {
      if (ticket > 0) {
        const Ticket& t = find_ticket(s, ticket);
        return t.info.state == DRGB_JOB_DONE || t.info.state == DRGB_JOB_FAILED;
      }
      return s->queue.empty() && s->by_batch_id.empty() && !s->stepping;
    };
    if (ticket > 0) find_ticket(s, ticket);
    if (timeout_s < 0) {
      s->cv_done.wait(lk, done);
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
      throw CudaError("timed out waiting for the job", DRGB_ERR_STATE);
    }
  });
}

int drgb_server_job_info(drgb_server* s, int32_t ticket, drgb_job_info* out) {
  return guard([&] {
    require(s && out, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = find_ticket(s, ticket).info;
  });
}

int drgb_server_job_losses(drgb_server* s, int32_t ticket, int64_t first, int64_t n, float* out) {
  return guard([&] {
    require(s && (out || n == 0), "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    const Ticket& t = find_ticket(s, ticket);
    require(t.info.state == DRGB_JOB_DONE, "job not finished", DRGB_ERR_STATE);
    require(first >= 0 && n >= 0 && first + n <= (int64_t)t.losses.size(), "loss range beyond the iterations run");
    std::copy(t.losses.begin() + first, t.losses.begin() + first + n, out);
  });
}

int drgb_server_get_mesh(drgb_server* s, int32_t ticket, int mesh_id, float* vertices, float* colors,
                         float* texture, float* transforms) {
  return guard([&] {
    require(s != nullptr, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    const Ticket& t = find_ticket(s, ticket);
    require(t.info.state == DRGB_JOB_DONE, "job not finished", DRGB_ERR_STATE);
    require(mesh_id >= 0 && mesh_id < (int)t.out_v.size(), "mesh id out of range");
    if (vertices) std::copy(t.out_v[mesh_id].begin(), t.out_v[mesh_id].end(), vertices);
    if (colors) std::copy(t.out_col[mesh_id].begin(), t.out_col[mesh_id].end(), colors);
    if (texture) std::copy(t.out_tex[mesh_id].begin(), t.out_tex[mesh_id].end(), texture);
    if (transforms) std::copy(t.out_tr[mesh_id].begin(), t.out_tr[mesh_id].end(), transforms);
  });
}

int drgb_server_get_restricted(drgb_server* s, int32_t ticket, int mesh_id, float* params) {
  return guard([&] {
    require(s != nullptr && params != nullptr, "null server or output");
    std::lock_guard<std::mutex> lk(s->mu);
    const Ticket& t = find_ticket(s, ticket);
    require(t.info.state == DRGB_JOB_DONE, "job not finished", DRGB_ERR_STATE);
    require(mesh_id >= 0 && mesh_id < (int)t.out_rt.size(), "mesh id out of range");
    require(!t.out_rt[mesh_id].empty(), "not a restricted-transform mesh");
    std::copy(t.out_rt[mesh_id].begin(), t.out_rt[mesh_id].end(), params);
  });
}

int drgb_server_release(drgb_server* s, int32_t ticket) {
  return guard([&] {
    require(s != nullptr, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    const Ticket& t = find_ticket(s, ticket);
    require(t.info.state == DRGB_JOB_DONE || t.info.state == DRGB_JOB_FAILED, "job not finished", DRGB_ERR_STATE);
    s->tickets.erase(ticket);
  });
}

int drgb_server_get_stats(drgb_server* s, drgb_server_stats* out) {
  return guard([&] {
    require(s && out, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    drgb_server_stats st{};
    st.queued = (int32_t)s->queue.size();
    st.running = (int32_t)s->by_batch_id.size();
    st.done = s->n_done;
    st.failed = s->n_failed;
    st.bytes_in_use = s->bytes_in_use;
    st.bytes_budget = s->cfg.hbm_budget_bytes;
    st.bytes_peak = s->bytes_peak;
    st.batch_steps = s->batch_steps;
    st.job_iterations = s->job_iterations;
    st.busy_seconds = s->busy;
    st.now = s->now();
    *out = st;
  });
}

int drgb_server_step_times(drgb_server* s, int64_t first, int64_t n, float* ms, int32_t* jobs) {
  return guard([&] {
    require(s != nullptr, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    require(first >= 0 && n >= 0 && first + n <= (int64_t)s->step_ms.size(), "step range beyond the steps run");
    if (ms) std::copy(s->step_ms.begin() + first, s->step_ms.begin() + first + n, ms);
    if (jobs) std::copy(s->step_jobs.begin() + first, s->step_jobs.begin() + first + n, jobs);
  });
}

}  // extern "C"
