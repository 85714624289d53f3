// The renderer object behind the C ABI and the error-reporting helpers
// shared by the C-ABI translation units.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "engine.h"

namespace drgb {
void add_launches(int64_t n);
}  // namespace drgb

// Records / returns the message returned by drgb_last_error on this thread.
void drgb_set_last_error(const std::string& m);
std::string t_err_message();

template <class F>
static int guard(F&& f) {
  using namespace drgb;
  try {
    f();
    return DRGB_OK;
  } catch (const CudaError& e) {
    drgb_set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    drgb_set_last_error("host allocation failed");
    return DRGB_ERR_OOM;
  } catch (const std::exception& e) {
    drgb_set_last_error(e.what());
    return DRGB_ERR_INVALID;
  }
}

static inline void require(bool c, const char* msg, int code = DRGB_ERR_INVALID) {
  if (!c) throw drgb::CudaError(msg, code);
}

using namespace drgb;

struct drgb_renderer {
  int device = 0;
  cudaStream_t stream = nullptr;
  Job job;
  DevBuf<JobDev> d_job;
  DevBuf<int4> d_items;
  DevBuf<int> d_counter;
  DevBuf<CamDev> d_cam1;
  DevBuf<float> d_xy;
  DevBuf<uint32_t> d_u32;
  DevBuf<float> d_f32;
  int sm_count = 1;
  int use_graph = 1;
  cudaGraphExec_t graph = nullptr;
  int64_t graph_kernels = 0;
  bool graph_valid = false;

  // Side branch of an iteration: the edge pass's projection, pmf and CDF run
  // beside the pixel kernel when the mesh has many edges (the CDF is one
  // sequential chain per view).
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // Host-pointer calls copy the targets on `xfer` while the raster pass runs;
  // pixels_wait (when set) is the event the pixel kernel waits for.
  cudaStream_t xfer = nullptr;
  cudaEvent_t ev_xfer_fork = nullptr, ev_xfer = nullptr;
  cudaEvent_t pixels_wait = nullptr;
  int px_resident = 0;  // pixel blocks per SM of the current model (0: not queried)
  // Page-locked words a call reads back at its end in one wait: the kernels'
  // error flags, the tile lists' state, the light cells' overflow flag and
  // the loss.
  HostBuf<uint32_t> h_status;

  ~drgb_renderer() {
    if (graph) cudaGraphExecDestroy(graph);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_xfer_fork) cudaEventDestroy(ev_xfer_fork);
    if (ev_xfer) cudaEventDestroy(ev_xfer);
    if (xfer) cudaStreamDestroy(xfer);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
  }

  void set_device() const { DRGB_CUDA(cudaSetDevice(device)); }
  void require_commit() const { require(job.committed, "no scene committed (call drgb_commit first)", DRGB_ERR_STATE); }
  int px_blocks_per_sm = 8, edge_blocks_per_sm = 8;  // persistent grids (autotuned or set by option)
  int bvh_rebuild = 100;  // optimiser iterations between hierarchy rebuilds (0: refit only)
  int px_grid() const { return sm_count * px_blocks_per_sm; }
  int edge_grid() const { return sm_count * edge_blocks_per_sm; }

  // Pixel work items for the current views: view-major, tiles row-major.
  void make_items() {
    Job& J = job;
    std::vector<int4> items;
    for (int v = 0; v < J.n_views; v++) {
      const int W = (int)J.h_cams[v].width, H = (int)J.h_cams[v].height;
      for (int y = 0; y < H; y += J.tile_h)
        for (int x = 0; x < W; x += J.tile_w) items.push_back(make_int4(0, v, x, y));
    }
    J.h_pixel_items = items;
    d_items.upload(items.data(), items.size(), stream);
    J.loss_part.reserve(std::max<size_t>(1, items.size()));
    J.loss_blk.reserve((size_t)std::max(1, J.n_views) * kLossBlocks);
    if (!J.loss_ticket.p) {
      J.loss_ticket.alloc(1);
      DRGB_CUDA(cudaMemsetAsync(J.loss_ticket.p, 0, sizeof(unsigned), stream));
    }
    J.dev.item_base = 0;
    J.dev.item_count = (int)items.size();
  }

  // Views of the last call: repeated calls with the same cameras and tile
  // shape keep the device cameras and work items.
  std::vector<drgb_camera> last_cams;
  int last_tw = 0, last_th = 0;

  void views(const drgb_camera* cams, int n, bool same_size) {
    require(cams != nullptr && n > 0, "need at least one camera");
    if (same_size)
      for (int i = 1; i < n; i++)
        require((int)cams[i].width == (int)cams[0].width && (int)cams[i].height == (int)cams[0].height,
                "gradient calls need all views of the same size");
    if ((int)last_cams.size() == n && last_tw == job.tile_w && last_th == job.tile_h && d_items.p &&
        std::memcmp(last_cams.data(), cams, sizeof(drgb_camera) * (size_t)n) == 0)
      return;
    last_cams.clear();
    setup_views(job, cams, n);
    job.cams.upload(job.h_cams.data(), job.h_cams.size(), stream);
    std::vector<int64_t> off(n + 1, 0);
    for (int i = 0; i < n; i++) off[i + 1] = off[i] + (int64_t)cams[i].width * (int64_t)cams[i].height;
    job.img_off.upload(off.data(), off.size(), stream);
    make_items();
    last_cams.assign(cams, cams + n);
    last_tw = job.tile_w;
    last_th = job.tile_h;
  }

  int64_t n_pixels() const {
    int64_t s = 0;
    for (auto& c : job.h_cams) s += (int64_t)c.width * (int64_t)c.height;
    return s;
  }

  // Buffers of a gradient call over the current views.
  void gradient_buffers(int edge_samples) {
    Job& J = job;
    require(edge_samples >= 0, "edge sample count must be >= 0");
    const size_t npix = (size_t)J.n_views * J.W * J.H;
    J.adj.reserve(std::max<size_t>(1, npix));
    build_edges(J);
    J.proj.reserve(std::max<size_t>(1, (size_t)J.n_views * J.n_vertices));
    J.pmf.reserve(std::max<size_t>(1, (size_t)J.n_views * J.n_edges));
    J.cdf.reserve(std::max<size_t>(1, (size_t)J.n_views * (J.n_edges + 1)));
    J.queue.reserve(std::max<size_t>(1, (size_t)J.n_views * std::max(edge_samples, 1)));
#ifndef DRGB_EDGE_NO_SORT
    for (int b = 0; b < 2; b++) {
      J.qkey[b].reserve(J.queue.n);
      J.qidx[b].reserve(J.queue.n);
    }
    J.qhist.reserve(scan_scratch(256 * (size_t)kSortGrid));
    J.qn.reserve(1);
#endif
    J.dev.edge_samples = edge_samples;
    J.dev.rnd = edge_samples > 0 ? edge_random_table(edge_samples, stream) : nullptr;
    J.dev.rnd_order = edge_samples > 0 ? edge_random_order(edge_samples, stream) : nullptr;
    if (J.det) det_buffers(J, stream);
    if (J.store_hits) hit_buffers();
    raster_buffers();
  }

  // Rasterised primary visibility (DRGB_OPT_PRIMARY_RASTER) for the current
  // views: one 64-bit key per forward and per adjoint sample, the screen
  // tiles and their triangle lists.  raster_on tells sync_dev to hand the
  // buffers to the pixel kernel; call before push_dev.  Off for the
  // brute-force caster (the reference's loop, kept for parity) and for
  // stored adjoint hits.
  void raster_geometry(int& tw, int& th, int& ntx, int& nty) const {
    raster_tile(job.S, tw, th);
    int W = 1, H = 1;
    for (auto& c : job.h_cams) {
      W = std::max(W, (int)c.width);
      H = std::max(H, (int)c.height);
    }
    ntx = (W + tw - 1) / tw;
    nty = (H + th - 1) / th;
  }
  void raster_buffers() {
    Job& J = job;
    // Deterministic mode: a job runs its own raster pass alone, in a batch and
    // in the server, under the same size rule (the autotuner leaves the
    // choice to the rule), so the hits and the bits agree.  A call whose
    // lists overflow traces (and the lists grow for the next): traversal and
    // raster pass find the same hits except the reference caster's
    // clamped-determinant ones, which each finds only by chance.
    // Small calls: the raster pass's fixed cost (about 15 launches) outweighs
    // what it saves; measured on GB300, a 12-triangle cube at 256x256 x 16 spp
    // and 5,120 triangles at 512x512 x 4 spp x 2 views break even (1-2 M
    // samples).  Dense meshes: binning costs per (view, triangle) and the
    // tile lists grow long, so fewer than 32 forward samples per (view,
    // triangle) trace (GB300: 64 instances of 5,120 triangles, 4 views at
    // 512x512 x 16 spp, 13 samples, 0.88x; the 200k-triangle path-model
    // stress scene, 21 samples, 0.94x; point light from 51 samples on
    // 1.07-1.60x).  The optimiser's autotuner times both ways instead.
    const size_t samples = (size_t)n_pixels() * J.S;
    const bool pays = J.raster == 2 ? true
                      : J.raster_pick >= 0 ? J.raster_pick == 1 : raster_pays(samples, J.n_views, J.n_tris);
    const bool on = J.raster && pays && !J.trace_bruteforce && !J.store_hits && J.n_tris > 0 && J.n_views > 0;
    if (on) {
      J.vis[0].reserve(samples);
      J.vis[1].reserve(samples);
      if (vis_points(J.mode)) {
        J.vis_uv[0].reserve(samples);
        J.vis_uv[1].reserve(samples);
      }
      int tw, th, ntx, nty;
      raster_geometry(tw, th, ntx, nty);
      const size_t n_tiles = (size_t)J.n_views * ntx * nty;
      J.ra_tiles.reserve(scan_scratch(n_tiles + 1));
      J.ra_cursor.reserve(n_tiles);
      J.ra_state.reserve(1);
      J.ra_list.reserve(std::max<size_t>(1u << 16, (size_t)32 * J.n_views * J.n_tris));
      J.ra_rec.reserve((size_t)4 * J.n_views * J.n_tris);
    }
    J.raster_on = on;
    // point-light shadow rays (the models with the point light)
    const bool sh = on && (J.mode == LAMBERT_POINT_VCOLOR || J.mode == PATH_DIFFUSE);
    if (sh) {
      const int G = light_grid_size(J.n_tris);
      J.sh_grid.reserve(1);
      J.sh_cells.reserve(scan_scratch((size_t)G * G + 1));
      J.sh_cursor.reserve((size_t)G * G);
      J.sh_list.reserve(std::max<size_t>(1u << 16, (size_t)64 * J.n_tris));
      J.sh_rec.reserve((size_t)4 * J.n_tris);
    }
    J.shadow_on = sh;
  }

  // The raster pass for the samples a pixel-kernel launch with `flags`
  // traces (on `st` for the device job `dj`: the renderer's own by default,
  // a batch's copy of it otherwise).  Returns PX_VIS when it ran (add it to that launch's flags), 0
  // when the samples are to be traced: raster off, or the device job does
  // not hold the current, large enough buffers.
  int raster_pass(int flags, const JobDev* dj = nullptr, cudaStream_t st = nullptr) {
    Job& J = job;
    if (!dj) dj = d_job.p;
    if (!st) st = stream;
    const int passes = ((flags & PX_FWD) ? 1 : 0) | ((flags & PX_ADJ) ? 2 : 0);
    if (!J.raster_on || !passes) return 0;
    const size_t samples = (size_t)n_pixels() * J.S;
    int tw, th, ntx, nty;
    raster_geometry(tw, th, ntx, nty);
    const size_t n_tiles = (size_t)J.n_views * ntx * nty;
    if (J.dev.vis_fwd != J.vis[0].p || J.dev.vis_adj != J.vis[1].p || J.dev.ra_state != J.ra_state.p ||
        J.vis[0].n < samples || J.vis[1].n < samples || J.ra_tiles.n < scan_scratch(n_tiles + 1) ||
        J.ra_cursor.n < n_tiles || !J.ra_list.p || J.ra_rec.n < (size_t)4 * J.n_views * J.n_tris ||
        (vis_points(J.mode) && (J.dev.vis_uv_fwd != J.vis_uv[0].p || J.dev.vis_uv_adj != J.vis_uv[1].p ||
                                J.vis_uv[0].n < samples || J.vis_uv[1].n < samples))) {
      // nothing built for this call: no stale hit or list may be read either
      // (state 0x01010101: bit 0 "wrote nothing" set, bit 1 "lists valid" clear)
      if (J.ra_state.p) DRGB_CUDA(cudaMemsetAsync(J.ra_state.p, 1, sizeof(uint32_t), st));
      if (J.sh_grid.p) DRGB_CUDA(cudaMemsetAsync(J.sh_grid.p, 0, sizeof(LightGrid), st));
      return 0;
    }
    launch_raster(dj, J, passes, ntx, nty, tw, th, st);
    const int G = light_grid_size(J.n_tris);
    if (J.shadow_on && J.dev.sh_grid == J.sh_grid.p && J.sh_cells.n >= scan_scratch((size_t)G * G + 1) &&
        J.sh_cursor.n >= (size_t)G * G && J.sh_rec.n >= (size_t)4 * J.n_tris && J.sh_list.p)
      launch_light_grid(dj, J, G, st);
    else if (J.sh_grid.p)
      DRGB_CUDA(cudaMemsetAsync(J.sh_grid.p, 0, sizeof(LightGrid), st));
    return PX_VIS;
  }

  // After a synchronised call: lists that did not fit (state bit 0 of the
  // tile lists, the light cells' overflow flag, as check_flags read them
  // back) double their room for the next call (that call traced instead).
  void raster_grow(uint32_t tiles_state, uint32_t cells_overflow) {
    Job& J = job;
    if (tiles_state & 1u) {
      J.ra_list.alloc(2 * J.ra_list.n);
      DRGB_CUDA(cudaMemsetAsync(J.ra_state.p, 0, sizeof(uint32_t), stream));
      graph_valid = false;
      push_dev();
    }
    if (cells_overflow) {
      J.sh_list.alloc(2 * J.sh_list.n);
      DRGB_CUDA(cudaMemsetAsync(J.sh_grid.p, 0, sizeof(LightGrid), stream));
      graph_valid = false;
      push_dev();
    }
  }

  // One float4 per adjoint sample of every work item (stored-hit mode).
  void hit_buffers() {
    Job& J = job;
    const int64_t n = (int64_t)J.dev.item_count * J.tile_w * J.tile_h * J.S;
    J.hit_buf.reserve(std::max<int64_t>(1, n));
  }

  // The pixel kernel; with stored hits, an adjoint pass is preceded by a
  // launch that traces and stores the adjoint samples' primary hits.
  void pixel_pass(int flags) {
    Job& J = job;
    const bool hits = J.store_hits && J.hit_buf.p && (flags & PX_ADJ);
    const int n = (int)J.h_pixel_items.size();
    flags |= raster_pass(flags);
    wait_inputs();
    if (hits) launch_pixels(d_job.p, d_items.p, n, d_counter.p, PX_ADJ | PX_HIT_STORE, px_grid(), stream, J.mode, J.det);
    launch_pixels(d_job.p, d_items.p, n, d_counter.p, flags | (hits ? PX_HIT_LOAD : 0), px_grid(), stream, J.mode,
                  J.det);
  }

  // The pixel kernel reads the targets: wait for their copy (see xfer).
  void wait_inputs() {
    if (pixels_wait) DRGB_CUDA(cudaStreamWaitEvent(stream, pixels_wait, 0));
  }

  // Copies n bytes of host data to dst on the transfer stream, after the work
  // already on the renderer's stream (which may still read dst); the next
  // pixel pass waits for the copy, while the raster pass overlaps it.
  void upload_inputs(void* dst, const void* src, size_t n) {
    if (!xfer) {
      DRGB_CUDA(cudaStreamCreateWithFlags(&xfer, cudaStreamNonBlocking));
      DRGB_CUDA(cudaEventCreateWithFlags(&ev_xfer_fork, cudaEventDisableTiming));
      DRGB_CUDA(cudaEventCreateWithFlags(&ev_xfer, cudaEventDisableTiming));
    }
    DRGB_CUDA(cudaEventRecord(ev_xfer_fork, stream));
    DRGB_CUDA(cudaStreamWaitEvent(xfer, ev_xfer_fork, 0));
    DRGB_CUDA(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, xfer));
    DRGB_CUDA(cudaEventRecord(ev_xfer, xfer));
    pixels_wait = ev_xfer;
  }

  // Deterministic mode: clear the record counts before a gradient pass and
  // reduce the records into the gradient after it.
  void det_begin() {
    if (job.det && job.rec_key.p) launch_det_clear(job, stream);
  }
  void det_end() {
    if (job.det && job.rec_key.p) launch_det_reduce(job, sm_count, stream);
  }

  // images = false: the device copy writes no images (a call that returns
  // none), the host copy keeps the buffer.
  void push_dev(bool images = true) {
    JobDev keep = job.dev;
    sync_dev(job);
    job.dev.item_base = keep.item_base;
    job.dev.item_count = keep.item_count;
    job.dev.edge_samples = keep.edge_samples;
    job.dev.rnd = keep.rnd;
    job.dev.rnd_order = keep.rnd_order;
    d_job.alloc(1);
    JobDev d = job.dev;
    if (!images) d.images = nullptr;
    DRGB_CUDA(cudaMemcpyAsync(d_job.p, &d, sizeof(JobDev), cudaMemcpyHostToDevice, stream));
  }

  // The end of a call: one wait for the stream, then the kernels' error
  // flags (an error throws), the lists' overflow state, and (loss non-null)
  // the loss of the call copied to host memory.
  void check_flags(float* loss = nullptr) {
    Job& J = job;
    h_status.reserve(4);
    uint32_t* h = h_status.p;
    h[1] = h[2] = 0;
    DRGB_CUDA(cudaMemcpyAsync(h, J.err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    if (J.raster_on && J.ra_state.p)
      DRGB_CUDA(cudaMemcpyAsync(h + 1, J.ra_state.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    if (J.shadow_on && J.sh_grid.p)
      DRGB_CUDA(cudaMemcpyAsync(h + 2, reinterpret_cast<const char*>(J.sh_grid.p) + offsetof(LightGrid, overflow),
                                sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    if (loss) DRGB_CUDA(cudaMemcpyAsync(h + 3, J.loss_out.p, sizeof(float), cudaMemcpyDeviceToHost, stream));
    DRGB_CUDA(cudaStreamSynchronize(stream));
    if (loss) std::memcpy(loss, h + 3, sizeof(float));
    const uint32_t f = h[0];
    raster_grow(h[1], h[2]);
    if (f) {
      DRGB_CUDA(cudaMemsetAsync(job.err.p, 0, sizeof(uint32_t), stream));
      DRGB_CUDA(cudaStreamSynchronize(stream));
      std::string m = "kernel error flags " + std::to_string(f);
      if (f & ERR_STACK_OVERFLOW) m += " (traversal stack overflow)";
      if (f & ERR_TRAVERSAL_LIMIT) m += " (traversal step limit)";
      if (f & ERR_VISIBILITY) m += " (rasterised hit names a triangle the scene does not have)";
      throw CudaError(m, DRGB_ERR_KERNEL);
    }
  }

  // Work items of a new tile shape, with the buffers that depend on them.
  void apply_tile(int tw, int th) {
    job.tile_w = tw;
    job.tile_h = th;
    make_items();
    if (job.det && job.rec_key.p) det_buffers(job, stream);
    if (job.store_hits) hit_buffers();
    push_dev();
    graph_valid = false;
  }

  // Meshes with at least this many edges run the CDF beside the pixel pass.
  static constexpr int kSideCdfEdges = 50000;
  bool side_cdf() const {
#ifdef DRGB_NO_SIDE_CDF
    return false;
#endif
    return job.dev.edge_samples > 0 && job.n_edges >= kSideCdfEdges && !job.det && !job.store_hits;
  }

  // Forward + loss + interior adjoint + edges of the current views; grad is
  // cleared first.  Everything is enqueued on the stream (and, for meshes
  // with many edges, on the side stream that joins it before the edge
  // samples are drawn).
  void enqueue_iteration(bool want_images) {
    Job& J = job;
    const bool interior = J.mode != SILHOUETTE;
    DRGB_CUDA(cudaMemsetAsync(J.grad.p, 0, J.grad_bytes(), stream));
    det_begin();
    int flags = PX_FWD | PX_LOSS | (interior ? PX_ADJ : 0) | (want_images ? PX_IMG : 0);
    if (side_cdf()) {
      if (!side) {
        DRGB_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
        DRGB_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        DRGB_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
      }
      if (!px_resident) px_resident = pixel_blocks_resident(J.mode);
      DRGB_CUDA(cudaEventRecord(ev_fork, stream));
      DRGB_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
      launch_edges_prep(d_job.p, 0, J.n_edges, J.n_views, J.n_vertices, side);
      DRGB_CUDA(cudaEventRecord(ev_join, side));
      // one SM slot per CDF block stays free of the persistent pixel kernel
      const int grid = std::max(1, std::min(px_grid(), sm_count * px_resident - J.n_views));
      flags |= raster_pass(flags);
      wait_inputs();
      launch_pixels(d_job.p, d_items.p, (int)J.h_pixel_items.size(), d_counter.p, flags, grid, stream, J.mode, J.det);
      launch_loss_finalize(d_job.p, 1, stream);
      DRGB_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
      launch_edges_rest(d_job.p, 0, J.n_edges, J.n_views, J.dev.edge_samples, J.queue_count.p, edge_grid(), stream,
                        false, &J, J.mode);
    } else {
      pixel_pass(flags);
      launch_loss_finalize(d_job.p, 1, stream);
      if (J.dev.edge_samples > 0) launch_edges(d_job.p, 0, J, edge_grid(), stream);
    }
    det_end();
    launch_restricted_grad(J, stream);
  }
};

