// C ABI of the renderer (include/drgb.h).  Each drgb_renderer owns one job
// (scene, LBVH, views, gradient and optimiser state) and one CUDA stream.
// Errors never escape as exceptions: they become negative return codes
// with a per-thread message (drgb_last_error).
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <memory>
#include <string>

#include "renderer.h"

namespace drgb {
static std::atomic<int64_t> g_launches{0};
static thread_local int64_t t_capture_count = 0;
static thread_local bool t_capturing = false;
void count_launch(int n) {
  if (t_capturing) t_capture_count += n;
  else g_launches += n;
}
void add_launches(int64_t n) { g_launches += n; }
}  // namespace drgb

static thread_local std::string t_err;
void drgb_set_last_error(const std::string& m) { t_err = m; }
std::string t_err_message() { return t_err; }

static void check_renderer(drgb_renderer* r) { require(r != nullptr, "null renderer"); }

namespace drgb {
void launch_rs_scan(uint32_t* hist, int m, cudaStream_t s);
}  // namespace drgb

extern "C" {

int drgb_abi_version(void) { return DRGB_ABI_VERSION; }

int drgb_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return DRGB_ERR_INVALID;
  std::snprintf(buf, len, "%s", t_err.c_str());
  return DRGB_OK;
}

int64_t drgb_kernel_launches(void) { return g_launches.load(); }

int drgb_debug_exclusive_scan(const uint32_t* counts, int n, uint32_t* out) {
  return guard([&] {
    require(counts && out && n >= 1, "null array or empty scan");
    DevBuf<uint32_t> d;
    d.alloc(scan_scratch((size_t)n));
    DRGB_CUDA(cudaMemcpy(d.p, counts, sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    launch_rs_scan(d.p, n, 0);
    DRGB_CUDA(cudaGetLastError());
    DRGB_CUDA(cudaMemcpy(out, d.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
  });
}

int drgb_camera_look_at(const float origin[3], const float target[3], const float up[3], float width, float height,
                        float fov_rad, float znear, float zfar, drgb_camera* out) {
  return guard([&] {
    require(origin && target && up && out, "null argument");
    camera_look_at(origin, target, up, width, height, fov_rad, znear, zfar, out);
  });
}

int drgb_renderer_create(int shading_model, int spp, int device, drgb_renderer** out) {
  return guard([&] {
    require(out != nullptr, "null output pointer");
    *out = nullptr;
    switch (shading_model) {
      case DRGB_SILHOUETTE: case DRGB_VERTEX_COLOR: case DRGB_TEXTURE_COLOR: case DRGB_LAMBERT: case DRGB_PHONG:
      case DRGB_GGX: case DRGB_PATH_TEST:
      case DRGB_LAMBERT_POINT_VCOLOR: case DRGB_PATH_DIFFUSE: break;
      default: throw CudaError("unknown shading model " + std::to_string(shading_model), DRGB_ERR_UNSUPPORTED);
    }
    require(spp >= 1 && spp <= 64, "spp must be in [1, 64]");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw CudaError("no CUDA device", DRGB_ERR_NO_DEVICE);
    require(device >= 0 && device < n, "device index out of range");
    auto r = std::make_unique<drgb_renderer>();
    r->device = device;
    DRGB_CUDA(cudaSetDevice(device));
    DRGB_CUDA(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
    DRGB_CUDA(cudaDeviceGetAttribute(&r->sm_count, cudaDevAttrMultiProcessorCount, device));
    init_job_model(r->job, shading_model, spp);
    r->d_counter.alloc(1);
    *out = r.release();
  });
}

int drgb_renderer_destroy(drgb_renderer* r) {
  if (!r) return DRGB_ERR_INVALID;
  return guard([&] {
    cudaSetDevice(r->device);
    cudaStreamSynchronize(r->stream);
    delete r;
  });
}

void* drgb_renderer_stream(drgb_renderer* r) { return r ? (void*)r->stream : nullptr; }

int drgb_renderer_set_option(drgb_renderer* r, int option, int64_t value) {
  return guard([&] {
    check_renderer(r);
    switch (option) {
      case DRGB_OPT_TRACE_BRUTEFORCE: r->job.trace_bruteforce = value ? 1 : 0; break;
      case DRGB_OPT_TILE_W:
      case DRGB_OPT_TILE_H: {
        const int v = (int)value;
        require(v >= 1, "tile size must be >= 1");
        const int tw = option == DRGB_OPT_TILE_W ? v : r->job.tile_w;
        const int th = option == DRGB_OPT_TILE_H ? v : r->job.tile_h;
        require(tw * th <= 32 && tw * th * r->job.S <= 64, "a tile holds at most 32 pixels and 64 samples");
        r->job.tile_w = tw;
        r->job.tile_h = th;
        break;
      }
      case DRGB_OPT_USE_GRAPH: r->use_graph = value ? 1 : 0; break;
      case DRGB_OPT_BVH_BUILDER:
        require(value >= 0 && value <= 3,
                "hierarchy builder: 0 (LBVH), 1 (binned SAH, two-level when instanced), 2 (two-level), 3 (flat SAH)");
        r->job.bvh_builder = (int)value;  // used from the next commit on
        break;
      case DRGB_OPT_BVH_REBUILD:
        require(value >= 0 && value <= (1 << 30), "hierarchy rebuild period: 0 (never) or iterations");
        r->bvh_rebuild = (int)value;
        break;
      case DRGB_OPT_PIXEL_GRID:
        require(value >= 1 && value <= 64, "pixel grid: 1..64 blocks per SM");
        r->px_blocks_per_sm = (int)value;
        break;
      case DRGB_OPT_EDGE_GRID:
        require(value >= 1 && value <= 64, "edge grid: 1..64 blocks per SM");
        r->edge_blocks_per_sm = (int)value;
        break;
      case DRGB_OPT_ADJOINT_HITS: {
        Job& J = r->job;
        J.store_hits = value ? 1 : 0;
        if (J.store_hits && J.opt.active) {
          r->set_device();
          r->hit_buffers();
        }
        if (r->d_job.p) r->push_dev();
        break;
      }
      case DRGB_OPT_DETERMINISTIC: {
        Job& J = r->job;
        J.det = value ? 1 : 0;
        J.dev.det = 0;
        // an initialised optimiser gets its record buffers now; other calls
        // allocate them with their per-call buffers
        if (J.det && J.opt.active) {
          r->set_device();
          det_buffers(J, r->stream);
        }
        if (r->d_job.p) r->push_dev();
        break;
      }
      case DRGB_OPT_TRACE_STEP_LIMIT:
        require(value >= 0 && value <= (1 << 24), "traversal step limit: 1..16777216 (0: the default, 16777216)");
        r->job.trace_limit = value ? (int)value : (1 << 24);
        if (r->d_job.p) r->push_dev();
        break;
      case DRGB_OPT_EDGE_JACOBIAN:
        require(value == 0 || value == 1, "edge Jacobian: 0 (the reference's edge_grad) or 1 (full 2x3)");
        r->job.edge_exact = (int)value;
        if (r->d_job.p) r->push_dev();
        break;
      case DRGB_OPT_PRIMARY_RASTER:
        require(value >= 0 && value <= 2,
                "camera and shadow rays: 0 (hierarchy traversal), 1 (tiles and cells where that pays), 2 (always)");
        r->job.raster = (int)value;
        r->job.raster_pick = -1;
        if (r->d_job.p && r->job.n_views > 0) {
          r->raster_buffers();
          r->push_dev();
        }
        break;
      case DRGB_OPT_EDGE_SET:
        require(value == 0 || value == 1, "edge set: 0 (every edge, the reference's) or 1 (silhouette edges)");
        r->job.edge_sil = (int)value;
        if (r->d_job.p) r->push_dev();
        break;
      default: throw CudaError("unknown option", DRGB_ERR_INVALID);
    }
    // the raster pass depends on the caster, stored hits and deterministic mode
    if ((option == DRGB_OPT_TRACE_BRUTEFORCE || option == DRGB_OPT_DETERMINISTIC ||
         option == DRGB_OPT_ADJOINT_HITS) && r->d_job.p && r->job.n_views > 0) {
      r->set_device();
      r->raster_buffers();
      r->push_dev();
    }
    r->graph_valid = false;
  });
}

int drgb_renderer_set_model_params(drgb_renderer* r, const drgb_model_params* p) {
  return guard([&] {
    check_renderer(r);
    require(p != nullptr, "null params");
    for (int i = 0; i < 3; i++) r->job.mp.light_pos[i] = p->light_pos[i];
    r->job.mp.light_intensity = p->light_intensity;
    r->job.mp.ambient = p->ambient;
    r->job.mp.path_depth = std::max(0, std::min(16, (int)p->path_depth));
    r->job.mp.seed = p->seed;
    r->graph_valid = false;
  });
}

// Whether a cudaMemcpyAsync from host pointer p may read p after it returns:
// page-locked (and device) memory is read by the copy engine in stream
// order, pageable memory is staged before the call returns.
static bool read_after_return(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return true;
  }
  return a.type != cudaMemoryTypeUnregistered;
}

// Returns once the caller's arrays have been read: at once for pageable
// memory (the flattening and refit run on in stream order, ahead of the next
// call's work), after the stream has drained when an array is page-locked.
int drgb_commit(drgb_renderer* r, const drgb_scene_desc* scene) {
  return guard([&] {
    check_renderer(r);
    r->set_device();
    Job& J = r->job;
    upload_scene(J, scene, r->stream);
    J.opt.active = false;
    r->graph_valid = false;
    set_dscene(J, nullptr, 0, r->stream);
    commit_scene(J, r->stream);
    bool wait = false;
    for (int m = 0; m < scene->n_meshes && !wait; m++) {
      const drgb_mesh_desc& d = scene->meshes[m];
      for (const void* p : {(const void*)d.vertices, (const void*)d.colors, (const void*)d.tc,
                            (const void*)d.normals, (const void*)d.tangents, (const void*)d.indices,
                            (const void*)d.restricted, (const void*)d.texture})
        wait = wait || read_after_return(p);
    }
    if (wait) DRGB_CUDA(cudaStreamSynchronize(r->stream));
  });
}

int drgb_render(drgb_renderer* r, const drgb_camera* cams, int n_views, float* images) {
  return guard([&] {
    check_renderer(r);
    r->require_commit();
    require(images != nullptr, "null image buffer");
    r->set_device();
    Job& J = r->job;
    r->views(cams, n_views, false);
    const int64_t npx = r->n_pixels();
    J.images.reserve(3 * (size_t)npx);
    r->raster_buffers();
    r->push_dev();
    const int vis = r->raster_pass(PX_FWD);
    launch_pixels(r->d_job.p, r->d_items.p, (int)J.h_pixel_items.size(), r->d_counter.p, PX_FWD | PX_IMG | vis,
                  r->px_grid(), r->stream, J.mode);
    DRGB_CUDA(cudaMemcpyAsync(images, J.images.p, sizeof(float) * 3 * npx, cudaMemcpyDeviceToHost, r->stream));
    r->check_flags();
  });
}

int drgb_dscene_layout(drgb_renderer* r, const int32_t* ids, int n_ids, int32_t* layout, int64_t* total) {
  return guard([&] {
    check_renderer(r);
    r->require_commit();
    std::vector<DLayout> L;
    const int64_t t = compute_layout(r->job, ids, n_ids, L);
    if (layout)
      for (size_t k = 0; k < L.size(); k++) {
        int32_t* o = layout + 9 * k;
        o[0] = L[k].vertices; o[1] = L[k].instances; o[2] = L[k].pos_off; o[3] = L[k].color_off;
        o[4] = L[k].tex_off; o[5] = L[k].rt_off >= 0 ? -1 : L[k].tr_off; o[6] = L[k].rt_off; o[7] = L[k].full;
        o[8] = L[k].mesh_id;
      }
    if (total) *total = t;
  });
}

int drgb_d_render(drgb_renderer* r, const drgb_camera* cams, const float* adjoints, int n_views,
                  int edge_samples_in_total, const int32_t* ids, int n_ids, float* dscene) {
  return guard([&] {
    check_renderer(r);
    r->require_commit();
    require(adjoints && dscene, "null adjoint or gradient buffer");
    r->set_device();
    Job& J = r->job;
    r->views(cams, n_views, true);
    set_dscene(J, ids, n_ids, r->stream);
    r->gradient_buffers(edge_samples_in_total);
    const size_t npix = (size_t)n_views * J.W * J.H;
    J.adj_in.reserve(3 * npix);
    DRGB_CUDA(cudaMemcpyAsync(J.adj_in.p, adjoints, sizeof(float) * 3 * npix, cudaMemcpyHostToDevice, r->stream));
    if (J.grad_total > 0)
      DRGB_CUDA(cudaMemcpyAsync(J.grad.p, dscene, sizeof(float) * J.grad_total, cudaMemcpyHostToDevice, r->stream));
    if (J.grad_alloc > J.grad_total)
      DRGB_CUDA(cudaMemsetAsync(J.grad.p + J.grad_total, 0, sizeof(float) * (J.grad_alloc - J.grad_total), r->stream));
    r->push_dev();
    launch_adj_convert(r->d_job.p, (int64_t)npix, r->stream);
    r->det_begin();
    if (J.mode != SILHOUETTE) r->pixel_pass(PX_ADJ);
    if (edge_samples_in_total > 0) launch_edges(r->d_job.p, 0, J, r->edge_grid(), r->stream);
    r->det_end();
    launch_restricted_grad(J, r->stream);
    if (J.grad_total > 0)
      DRGB_CUDA(cudaMemcpyAsync(dscene, J.grad.p, sizeof(float) * J.grad_total, cudaMemcpyDeviceToHost, r->stream));
    r->check_flags();
  });
}

static void d_render_and_compare_impl(drgb_renderer* r, const drgb_camera* cams, const float* targets, int n_views,
                                      int edge_samples, const int32_t* ids, int n_ids, float* dscene,
                                      float* out_images, float* loss, bool device_ptrs) {
  check_renderer(r);
  r->require_commit();
  require(targets && dscene, "null target or gradient buffer");
  r->set_device();
  Job& J = r->job;
  r->views(cams, n_views, true);
  set_dscene(J, ids, n_ids, r->stream);
  r->gradient_buffers(edge_samples);
  const size_t npix = (size_t)n_views * J.W * J.H;
  const cudaMemcpyKind h2d = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind d2h = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  J.targets.reserve(3 * npix);
  if (device_ptrs) DRGB_CUDA(cudaMemcpyAsync(J.targets.p, targets, sizeof(float) * 3 * npix, h2d, r->stream));
  else r->upload_inputs(J.targets.p, targets, sizeof(float) * 3 * npix);
  if (out_images) J.images.reserve(3 * npix);
  r->push_dev(out_images != nullptr);  // images are only written when requested
  r->enqueue_iteration(out_images != nullptr);
  if (r->pixels_wait) {  // a pass without pixel kernel (no views) still orders the copy
    DRGB_CUDA(cudaStreamWaitEvent(r->stream, r->pixels_wait, 0));
    r->pixels_wait = nullptr;
  }
  if (J.grad_total > 0) DRGB_CUDA(cudaMemcpyAsync(dscene, J.grad.p, sizeof(float) * J.grad_total, d2h, r->stream));
  if (out_images)
    DRGB_CUDA(cudaMemcpyAsync(out_images, J.images.p, sizeof(float) * 3 * npix, d2h, r->stream));
  if (device_ptrs) {
    if (loss) DRGB_CUDA(cudaMemcpyAsync(loss, J.loss_out.p, sizeof(float), d2h, r->stream));
    DRGB_CUDA(cudaStreamSynchronize(r->stream));
  } else {
    r->check_flags(loss);  // the loss comes back with the status words, in the call's one wait
  }
}

int drgb_d_render_and_compare(drgb_renderer* r, const drgb_camera* cams, const float* targets, int n_views,
                              int edge_samples, const int32_t* ids, int n_ids, float* dscene, float* out_images,
                              float* loss) {
  return guard([&] {
    d_render_and_compare_impl(r, cams, targets, n_views, edge_samples, ids, n_ids, dscene, out_images, loss, false);
  });
}

int drgb_d_render_and_compare_device(drgb_renderer* r, const drgb_camera* cams, const float* d_targets, int n_views,
                                     int edge_samples, const int32_t* ids, int n_ids, float* d_dscene,
                                     float* d_out_images, float* d_loss) {
  return guard([&] {
    d_render_and_compare_impl(r, cams, d_targets, n_views, edge_samples, ids, n_ids, d_dscene, d_out_images, d_loss,
                              true);
  });
}

int drgb_cast_rays(drgb_renderer* r, const drgb_camera* cam, const float* xy, int64_t n, uint32_t* prim,
                   uint32_t* inst, uint32_t* geom, float* t, float* u, float* v) {
  return guard([&] {
    check_renderer(r);
    r->require_commit();
    require(cam && xy && prim && inst && geom && t && u && v && n >= 0, "null argument");
    r->set_device();
    if (n == 0) return;
    const CamDev c = make_cam(*cam);
    r->d_cam1.upload(&c, 1, r->stream);
    r->d_xy.upload(xy, 2 * (size_t)n, r->stream);
    r->d_u32.reserve(3 * (size_t)n);
    r->d_f32.reserve(3 * (size_t)n);
    r->push_dev();
    uint32_t* U = r->d_u32.p;
    float* F = r->d_f32.p;
    launch_cast(r->d_job.p, r->d_cam1.p, r->d_xy.p, n, U, U + n, U + 2 * n, F, F + n, F + 2 * n, r->stream);
    DRGB_CUDA(cudaMemcpyAsync(prim, U, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaMemcpyAsync(inst, U + n, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaMemcpyAsync(geom, U + 2 * n, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaMemcpyAsync(t, F, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaMemcpyAsync(u, F + n, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaMemcpyAsync(v, F + 2 * n, 4 * n, cudaMemcpyDeviceToHost, r->stream));
    r->check_flags();
  });
}

// ---- optimiser ----------------------------------------------------------------

int drgb_opt_params_default(int alg, drgb_opt_params* p) {
  return guard([&] {
    require(p != nullptr, "null params");
    std::memset(p, 0, sizeof(*p));
    p->alg = alg;
    p->decay_period = alg == DRGB_GD_ADAM ? 100 : 25;  // set_default, optimizer_simple.cpp:13-23
    p->decay_mult = 0.75f;
    p->base_lr = p->position_lr = p->textures_lr = p->transforms_lr = 0.1f;
    p->flags = DRGB_OPT_POS | DRGB_OPT_TFM | DRGB_OPT_COL | DRGB_OPT_TEX;
    p->n_dmesh_ids = 1;
    p->dmesh_ids[0] = 0;
  });
}

int drgb_optimizer_init(drgb_renderer* r, const drgb_scene_desc* scene, const drgb_camera* cams, const float* targets,
                        int n_views, const drgb_opt_params* p) {
  return guard([&] {
    check_renderer(r);
    require(scene && cams && targets && p, "null argument");
    require(p->alg >= DRGB_GD_NAIVE && p->alg <= DRGB_GD_ADAM, "unknown optimiser algorithm");
    require(p->n_dmesh_ids >= 1 && p->n_dmesh_ids <= 16, "need 1..16 differentiable meshes");
    r->set_device();
    Job& J = r->job;
    upload_scene(J, scene, r->stream);
    set_dscene(J, p->dmesh_ids, p->n_dmesh_ids, r->stream);
    commit_scene(J, r->stream);
    r->views(cams, n_views, true);
    const size_t npix = (size_t)n_views * J.W * J.H;
    J.targets.reserve(3 * npix);
    DRGB_CUDA(cudaMemcpyAsync(J.targets.p, targets, sizeof(float) * 3 * npix, cudaMemcpyHostToDevice, r->stream));
    // EvalFunction passes targets[0].width*height edge samples (optimizer_simple.cpp:241)
    r->gradient_buffers(J.W * J.H);
    OptState& O = J.opt;
    O.params = *p;
    O.active = true;
    O.host_iter = 0;
    O.m.alloc(std::max<int64_t>(1, J.grad_total));
    O.G.alloc(std::max<int64_t>(1, J.grad_total));
    DRGB_CUDA(cudaMemsetAsync(O.m.p, 0, sizeof(float) * O.m.n, r->stream));
    DRGB_CUDA(cudaMemsetAsync(O.G.p, 0, sizeof(float) * O.G.n, r->stream));
    std::vector<float> lr;
    for (size_t k = 0; k < J.dlay.size(); k++) {
      lr.push_back(p->position_lr);
      lr.push_back(p->base_lr);
      lr.push_back(p->textures_lr);
      lr.push_back(p->transforms_lr);
    }
    O.lr.upload(lr.data(), lr.size(), r->stream);
    const int zero = 0;
    O.iter.upload(&zero, 1, r->stream);
    O.losses.alloc(1024);
    r->push_dev();
    DRGB_CUDA(cudaStreamSynchronize(r->stream));
    r->graph_valid = false;
  });
}

static void enqueue_opt_iteration(drgb_renderer* r) {
  Job& J = r->job;
  r->enqueue_iteration(false);
  launch_opt_record(J, r->stream);
  launch_opt_step(J, r->stream);
  prepare_scene(J, r->stream);
}

// n optimiser iterations: graph replays, or the launches themselves.
static void enqueue_opt_iterations(drgb_renderer* r, int64_t n_iters) {
  {
    if (r->use_graph) {
      if (!r->graph_valid) {
        if (r->graph) {
          cudaGraphExecDestroy(r->graph);
          r->graph = nullptr;
        }
        cudaGraph_t g;
        t_capturing = true;
        t_capture_count = 0;
        DRGB_CUDA(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
        try {
          enqueue_opt_iteration(r);
        } catch (...) {
          cudaStreamEndCapture(r->stream, &g);
          t_capturing = false;
          throw;
        }
        DRGB_CUDA(cudaStreamEndCapture(r->stream, &g));
        t_capturing = false;
        r->graph_kernels = t_capture_count;
        DRGB_CUDA(cudaGraphInstantiate(&r->graph, g, 0));
        cudaGraphDestroy(g);
        r->graph_valid = true;
      }
      for (int64_t i = 0; i < n_iters; i++) DRGB_CUDA(cudaGraphLaunch(r->graph, r->stream));
      add_launches(r->graph_kernels * n_iters);
    } else {
      for (int64_t i = 0; i < n_iters; i++) enqueue_opt_iteration(r);
    }
  }
}

int drgb_optimizer_run_async(drgb_renderer* r, int64_t n_iters) {
  return guard([&] {
    check_renderer(r);
    require(r->job.opt.active, "optimiser not initialised", DRGB_ERR_STATE);
    require(n_iters >= 0, "negative iteration count");
    r->set_device();
    Job& J = r->job;
    OptState& O = J.opt;
    const int64_t need = O.host_iter + n_iters;
    if ((int64_t)O.losses.n < need) {
      size_t cap = O.losses.n;
      while ((int64_t)cap < need) cap *= 2;
      DevBuf<float> nb;
      nb.alloc(cap);
      DRGB_CUDA(cudaMemcpyAsync(nb.p, O.losses.p, sizeof(float) * O.losses.n, cudaMemcpyDeviceToDevice, r->stream));
      DRGB_CUDA(cudaStreamSynchronize(r->stream));
      O.losses = std::move(nb);
      r->graph_valid = false;
    }
    // Hierarchy rebuilds: after every `period` iterations a host SAH build
    // from the current vertices starts on a host thread, behind the enqueued
    // iterations; `period / 2` iterations later its topology is copied in
    // (waiting for the build if needed).  The device pointers stay the same,
    // so the captured graph stays valid, and the iteration at which a
    // topology takes over depends only on the iteration count, not on timing.
    const int64_t period = r->bvh_rebuild, lag = period / 2;
    while (n_iters > 0) {
      int64_t n = n_iters;
      if (period > 0) {
        const int64_t ph = O.host_iter % period;
        n = std::min<int64_t>(n, ph < lag ? lag - ph : period - ph);
      }
      enqueue_opt_iterations(r, n);
      O.host_iter += n;
      n_iters -= n;
      if (period > 0) {
        const int64_t ph = O.host_iter % period;
        if (ph == 0) rebuild_bvh_start(J, r->stream);
        if (ph == lag) rebuild_bvh_apply(J, r->stream);
      }
    }
  });
}


int drgb_optimizer_run(drgb_renderer* r, int64_t n_iters, float* final_error, float* losses) {
  const int64_t start = r ? r->job.opt.host_iter : 0;
  int rc = drgb_optimizer_run_async(r, n_iters);
  if (rc != DRGB_OK) return rc;
  return guard([&] {
    Job& J = r->job;
    std::vector<float> h((size_t)std::max<int64_t>(1, n_iters));
    if (n_iters > 0)
      DRGB_CUDA(cudaMemcpyAsync(h.data(), J.opt.losses.p + start, sizeof(float) * n_iters, cudaMemcpyDeviceToHost,
                                r->stream));
    r->check_flags();
    if (losses && n_iters > 0) std::memcpy(losses, h.data(), sizeof(float) * n_iters);
    if (final_error && n_iters > 0) *final_error = h[n_iters - 1];
  });
}

int drgb_optimizer_profile(drgb_renderer* r, int n_iters, float* out_ms) {
  return guard([&] {
    check_renderer(r);
    require(r->job.opt.active, "optimiser not initialised", DRGB_ERR_STATE);
    require(n_iters >= 1 && out_ms, "bad arguments");
    r->set_device();
    Job& J = r->job;
    cudaEvent_t ev[5];
    for (auto& e : ev) DRGB_CUDA(cudaEventCreate(&e));
    double acc[5] = {0, 0, 0, 0, 0};
    for (int it = 0; it < n_iters; it++) {
      DRGB_CUDA(cudaEventRecord(ev[0], r->stream));
      DRGB_CUDA(cudaMemsetAsync(J.grad.p, 0, J.grad_bytes(), r->stream));
      r->det_begin();
      const int flags = PX_FWD | PX_LOSS | (J.mode != SILHOUETTE ? PX_ADJ : 0);
      r->pixel_pass(flags);
      launch_loss_finalize(r->d_job.p, 1, r->stream);
      DRGB_CUDA(cudaEventRecord(ev[1], r->stream));
      if (J.dev.edge_samples > 0) launch_edges(r->d_job.p, 0, J, r->edge_grid(), r->stream);
      r->det_end();  // deterministic mode: the record reduction is timed with the edge phase
      launch_restricted_grad(J, r->stream);
      DRGB_CUDA(cudaEventRecord(ev[2], r->stream));
      launch_opt_record(J, r->stream);
      launch_opt_step(J, r->stream);
      DRGB_CUDA(cudaEventRecord(ev[3], r->stream));
      prepare_scene(J, r->stream);
      DRGB_CUDA(cudaEventRecord(ev[4], r->stream));
      DRGB_CUDA(cudaEventSynchronize(ev[4]));
      float ms;
      for (int k = 0; k < 4; k++) {
        DRGB_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
        acc[k] += ms;
      }
      DRGB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[4]));
      acc[4] += ms;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    J.opt.host_iter += n_iters;
    for (int k = 0; k < 5; k++) out_ms[k] = (float)(acc[k] / n_iters);
    r->check_flags();
  });
}

// Mean device time (ms) of `iters` gradient passes (forward, loss, interior
// adjoint, edges) of the optimiser's views, without the update: the
// optimiser's state does not change.
static float time_gradient_passes(drgb_renderer* r, int iters) {
  cudaEvent_t e0, e1;
  DRGB_CUDA(cudaEventCreate(&e0));
  DRGB_CUDA(cudaEventCreate(&e1));
  r->enqueue_iteration(false);  // warm-up
  DRGB_CUDA(cudaEventRecord(e0, r->stream));
  for (int i = 0; i < iters; i++) r->enqueue_iteration(false);
  DRGB_CUDA(cudaEventRecord(e1, r->stream));
  DRGB_CUDA(cudaEventSynchronize(e1));
  float ms = 0.0f;
  DRGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / iters;
}

int drgb_optimizer_autotune(drgb_renderer* r, int trial_iters, int32_t* chosen, float* best_ms) {
  return guard([&] {
    check_renderer(r);
    require(r->job.opt.active, "optimiser not initialised", DRGB_ERR_STATE);
    require(trial_iters >= 1, "trial_iters must be >= 1");
    r->set_device();
    Job& J = r->job;
    const int S = J.S;
    float best = 1e30f;
    // 0. camera samples and point-light shadow rays by the raster pass or by
    //    traversal (the raster pass has a fixed cost that small calls do not
    //    recover); deterministic mode keeps the size rule, which the job
    //    follows alone, in a batch and in the server alike
    if (J.raster == 1 && !J.det && !J.trace_bruteforce && !J.store_hits) {
      int pick = 1;
      for (int k : {0, 1}) {
        J.raster_pick = k;
        r->raster_buffers();
        r->push_dev();
        r->graph_valid = false;
        const float ms = time_gradient_passes(r, trial_iters);
        if (ms < best) {
          best = ms;
          pick = k;
        }
      }
      J.raster_pick = pick;
      r->raster_buffers();
      r->push_dev();
    }
    // 1. work-item shape: 32 or 64 samples (one or two warp passes), at most 32 pixels
    std::vector<std::pair<int, int>> tiles;
    for (int n_samples : {32, 64}) {
      const int P = std::max(1, std::min(32, n_samples / std::max(1, S)));
      for (int th = 1; th * th <= P; th *= 2)
        if (P % th == 0 && P / th >= th) tiles.emplace_back(P / th, th);
    }
    int bw = J.tile_w, bh = J.tile_h;
    for (auto [tw, th] : tiles) {
      r->apply_tile(tw, th);
      const float ms = time_gradient_passes(r, trial_iters);
      if (ms < best) {
        best = ms;
        bw = tw;
        bh = th;
      }
    }
    r->apply_tile(bw, bh);
    // 2. persistent grid of the pixel kernel, 3. of the edge-shading kernel
    for (int which = 0; which < 2; which++) {
      int& knob = which == 0 ? r->px_blocks_per_sm : r->edge_blocks_per_sm;
      int bk = knob;
      for (int k : {2, 4, 8, 16}) {
        knob = k;
        const float ms = time_gradient_passes(r, trial_iters);
        if (ms < best) {
          best = ms;
          bk = k;
        }
      }
      knob = bk;
    }
    r->graph_valid = false;
    r->check_flags();
    if (chosen) {
      chosen[0] = J.tile_w;
      chosen[1] = J.tile_h;
      chosen[2] = r->px_blocks_per_sm;
      chosen[3] = r->edge_blocks_per_sm;
      chosen[4] = J.raster_on ? 1 : 0;
    }
    if (best_ms) *best_ms = best;
  });
}

int drgb_count_work(drgb_renderer* r, uint64_t* counts) {
  return guard([&] {
    check_renderer(r);
    r->require_commit();
    require(counts != nullptr, "null counts");
    require(r->job.n_views > 0 && r->job.targets.p, "run a gradient call or optimiser init first", DRGB_ERR_STATE);
    r->set_device();
    Job& J = r->job;
    DevBuf<unsigned long long> w;
    w.alloc(4);  // rays, box tests, triangle tests, footprint tests
    DRGB_CUDA(cudaMemsetAsync(w.p, 0, 4 * sizeof(unsigned long long), r->stream));
    JobDev d = J.dev;
    d.work = w.p;
    DRGB_CUDA(cudaMemcpyAsync(r->d_job.p, &d, sizeof(JobDev), cudaMemcpyHostToDevice, r->stream));
    const int flags = PX_FWD | PX_LOSS | (J.mode != SILHOUETTE ? PX_ADJ : 0);
    // gradients of this replay are discarded: save and restore the buffer
    DevBuf<float> save;
    save.alloc(std::max<int64_t>(1, J.grad_alloc));
    DRGB_CUDA(cudaMemcpyAsync(save.p, J.grad.p, save.bytes(), cudaMemcpyDeviceToDevice, r->stream));
    DRGB_CUDA(cudaMemsetAsync(J.grad.p, 0, save.bytes(), r->stream));
    const int vis = r->raster_pass(flags);  // its candidate tests count as rays and triangle tests
    launch_pixels(r->d_job.p, r->d_items.p, (int)J.h_pixel_items.size(), r->d_counter.p, flags | vis,
                  r->px_grid(), r->stream, J.mode);
    if (J.dev.edge_samples > 0) launch_edges(r->d_job.p, 0, J, r->edge_grid(), r->stream);
    int shaded = 0;
    DRGB_CUDA(cudaMemcpyAsync(&shaded, J.queue_count.p, sizeof(int), cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaMemcpyAsync(J.grad.p, save.p, save.bytes(), cudaMemcpyDeviceToDevice, r->stream));
    unsigned long long h[4];
    DRGB_CUDA(cudaMemcpyAsync(h, w.p, sizeof(h), cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaMemcpyAsync(r->d_job.p, &J.dev, sizeof(JobDev), cudaMemcpyHostToDevice, r->stream));
    DRGB_CUDA(cudaStreamSynchronize(r->stream));
    counts[0] = h[0];
    counts[1] = h[1];
    counts[2] = h[2];
    counts[3] = (uint64_t)std::max(0, shaded);
    counts[4] = h[3];
    r->check_flags();
  });
}

int drgb_optimizer_get_mesh(drgb_renderer* r, int mesh_id, float* vertices, float* colors, float* texture,
                            float* transforms) {
  return guard([&] {
    check_renderer(r);
    r->require_commit();
    require(mesh_id >= 0 && mesh_id < (int)r->job.meshes.size(), "mesh id out of range");
    r->set_device();
    const MeshState& M = r->job.meshes[mesh_id];
    if (vertices)
      DRGB_CUDA(cudaMemcpyAsync(vertices, M.vertices.p, sizeof(float) * 3 * M.nv, cudaMemcpyDeviceToHost, r->stream));
    if (colors && M.has_colors)
      DRGB_CUDA(cudaMemcpyAsync(colors, M.colors.p, sizeof(float) * 3 * M.nv, cudaMemcpyDeviceToHost, r->stream));
    if (texture && M.texture.p)
      DRGB_CUDA(cudaMemcpyAsync(texture, M.texture.p, M.texture.bytes(), cudaMemcpyDeviceToHost, r->stream));
    if (transforms)
      DRGB_CUDA(cudaMemcpyAsync(transforms, M.transforms.p, M.transforms.bytes(), cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaStreamSynchronize(r->stream));
  });
}

int drgb_optimizer_get_restricted(drgb_renderer* r, int mesh_id, float* params) {
  return guard([&] {
    check_renderer(r);
    r->require_commit();
    require(mesh_id >= 0 && mesh_id < (int)r->job.meshes.size(), "mesh id out of range");
    const MeshState& M = r->job.meshes[mesh_id];
    require(M.restricted, "not a restricted-transform mesh");
    require(params != nullptr, "null output");
    r->set_device();
    DRGB_CUDA(cudaMemcpyAsync(params, M.rparams.p, M.rparams.bytes(), cudaMemcpyDeviceToHost, r->stream));
    DRGB_CUDA(cudaStreamSynchronize(r->stream));
  });
}

}  // extern "C"
