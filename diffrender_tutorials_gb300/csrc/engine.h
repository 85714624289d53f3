// Host-side engine: device-resident state of one render job and the launch
// sequences over it.  A job is one committed scene (meshes, instances,
// textures), its LBVH, its views and its gradient/optimiser state.  Kernels
// take an array of jobs so that the same launch serves one job (the plain
// path) or many (the batched path).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <future>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/drgb.h"
#include "device.cuh"

namespace drgb {

struct CudaError : std::runtime_error {
  int code;
  CudaError(const std::string& m, int c) : std::runtime_error(m), code(c) {}
};

#define DRGB_CUDA(x)                                                                                  \
  do {                                                                                                \
    cudaError_t e_ = (x);                                                                             \
    if (e_ != cudaSuccess)                                                                            \
      throw ::drgb::CudaError(std::string(#x) + ": " + cudaGetErrorString(e_),                       \
                              e_ == cudaErrorMemoryAllocation ? DRGB_ERR_OOM : DRGB_ERR_CUDA);       \
  } while (0)

// Owning device allocation.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) { reset(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    reset();
    if (count == 0) return;
    DRGB_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
    n = count;
  }
  // grow-only allocation (keeps the pointer when large enough)
  void reserve(size_t count) {
    if (count <= n && p) return;
    alloc(count);
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) DRGB_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Uploads count values from h unless the device buffer holds exactly them
// already (`last`: the host copy of its previous upload); a commit of an
// unchanged scene copies none of the tables derived from it.
template <class T>
void upload_changed(DevBuf<T>& d, std::vector<T>& last, const T* h, size_t count, cudaStream_t s) {
  if (d.p && d.n == count && last.size() == count && std::memcmp(last.data(), h, sizeof(T) * count) == 0) return;
  d.upload(h, count, s);
  last.assign(h, h + count);
}

// Page-locked host buffer: copies to and from it run asynchronously.
template <class T>
struct HostBuf {
  T* p = nullptr;
  size_t n = 0;
  HostBuf() = default;
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
  void reserve(size_t count) {
    if (count <= n && p) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    DRGB_CUDA(cudaMallocHost((void**)&p, std::max<size_t>(1, count) * sizeof(T)));
    n = count;
  }
};

// A hierarchy rebuild that overlaps the device's work (batched jobs): the
// flattened positions are copied out behind the enqueued steps, a host
// thread builds the SAH topology, and the new topology is copied in and
// refitted in stream order a few steps later.
struct TopoRebuild {
  int stage = 0;  // 0 idle, 1 positions in flight, 2 topology being built, 3 an optimiser rebuild in progress
  cudaEvent_t ev = nullptr;
  int builder = 1;  // the host builder in use
  HostBuf<float4> pos, nodes;
  HostBuf<float> block_tr;
  HostBuf<int> perm, leaf_parent, node_parent;
  std::future<void> task;
  ~TopoRebuild() {
    if (task.valid()) task.wait();
    if (ev) cudaEventDestroy(ev);
  }
};

// Gradient layout of one differentiable mesh (DMesh, dmesh.h:35-85).
struct DLayout {
  int mesh_id = -1;
  int vertices = 0, instances = 0;
  int pos_off = 0, color_off = -1, tex_off = -1, tr_off = 0;
  // Restricted mesh: its 7 parameters per instance at rt_off (public part),
  // while tr_off points past the public vector, at a scratch block of 12
  // matrix entries per instance that the edge pass accumulates into and
  // launch_restricted_grad() folds through the Jacobian of to_mat.
  int rt_off = -1;
  int full = 0;
  int64_t base = 0;  // offset in the concatenated vector
};

// Count of kernels launched by this library (reported by drgb_kernel_launches).
void count_launch(int n = 1);

struct MeshState {
  int nv = 0, ni = 0, n_inst = 1;
  bool restricted = false;  // TransformR instances: rparams drive transforms
  DevBuf<float> vertices, colors, tc, normals, tangents, transforms, texture, rparams;
  std::vector<float> h_transforms;  // instance matrices as committed (column major)
  int tex_w = 0, tex_h = 0, tex_c = 0;
  bool has_colors = false, has_tc = false, has_normals = false, has_tangents = false;
  std::vector<uint32_t> h_indices;
};

struct OptState {
  bool active = false;
  drgb_opt_params params{};
  DevBuf<float> m, G;
  DevBuf<float> lr;       // per dmesh 4 lr values (pos, color, tex, transform)
  DevBuf<int> iter;       // device iteration counter
  DevBuf<float> losses;   // per-iteration loss history (ring)
  int64_t host_iter = 0;
};

struct Job {
  // model
  int mode = VERTEX_COLOR;
  int spp = 1, sq = 1, S = 1;
  ModelParams mp{};
  int trace_bruteforce = 0;
  int trace_limit = 1 << 24;  // node pops per ray (DRGB_OPT_TRACE_STEP_LIMIT)
  int edge_exact = 0;         // DRGB_OPT_EDGE_JACOBIAN
  int edge_sil = 0;           // DRGB_OPT_EDGE_SET
  int raster = 1;             // DRGB_OPT_PRIMARY_RASTER
  int raster_pick = -1;       // the optimiser's autotuner's choice (-1: none, the size rule decides)
  bool raster_on = false;     // raster buffers set up for the current views (see renderer::raster_buffers)
  DevBuf<float4> vis[2];              // rasterised visibility of forward / adjoint samples
  DevBuf<float2> vis_uv[2];           // their u, v where the records hold shading points
  DevBuf<uint32_t> ra_tiles;          // triangles per screen tile, then their offsets (scan)
  DevBuf<uint32_t> ra_cursor;         // per tile fill cursor
  DevBuf<uint32_t> ra_state;          // bit 0: the tile lists did not fit ra_list
  DevBuf<int> ra_list;                // per tile the (view, leaf) footprints that overlap it
  DevBuf<float4> ra_rec;              // per (view, leaf) its footprint (4 float4)
  bool shadow_on = false;             // light-space cells for point-light shadow rays (renderer::raster_buffers)
  DevBuf<LightGrid> sh_grid;
  DevBuf<uint32_t> sh_cells, sh_cursor;
  DevBuf<int> sh_list;
  DevBuf<float4> sh_rec;
  int tile_w = 4, tile_h = 4;
  // scene
  bool committed = false;
  std::vector<MeshState> meshes;
  int n_vertices = 0, n_tris = 0, n_blocks = 0;
  std::vector<BlockDev> h_blocks;
  DevBuf<float4> pos, orig, col, nrm;
  DevBuf<float4> tan;  // flattened tangents, PATH_TEST only
  DevBuf<float2> tc;
  DevBuf<int4> tri_v;
  DevBuf<BlockDev> blocks;
  DevBuf<MeshDev> meshdev;
  std::vector<MeshDev> h_meshdev;  // the table as last uploaded
  DevBuf<float> block_tr;  // 32 floats per block: transform, inverse-transpose
  DevBuf<int> vblock;      // block of each flattened vertex
  DevBuf<MeshSrc> src_tab;
  DevBuf<const float*> tr_tab;
  DevBuf<float> tr_inv0;   // inverse transforms of mesh 0 at the first commit
  // host copies of the tables above as last uploaded (upload_changed)
  std::vector<BlockDev> up_blocks;
  std::vector<int> up_vblock;
  std::vector<MeshSrc> up_src_tab;
  std::vector<const float*> up_tr_tab;
  std::vector<float> up_tr_inv0;
  // BVH
  DevBuf<float4> nodes, tri;
  DevBuf<float4> nodes4;   // 4-wide view of the binary hierarchy, refreshed after each refit
  DevBuf<int> perm, leaf_parent, node_parent, counters;
  DevBuf<int> leaf_of;  // triangle -> leaf slot (inverse of perm)
  DevBuf<uint32_t> sort_keys[2], sort_hist;
  DevBuf<int> sort_vals[2];
  DevBuf<float> bounds;
  int root = 0;
  // hierarchy builder (0: LBVH from Morton codes on the device, 1 (default):
  // binned SAH on the host, measured faster to traverse) and the topology cache: a commit of the same triangles with
  // the same builder keeps the topology and only refits the boxes
  int bvh_builder = 1;
  std::vector<int4> h_tri_v, topo_tri_v;
  int topo_builder = -1;
  // overlapped rebuild in progress (optimiser or batch); declared after what its host thread reads, so that
  // it is destroyed, and waits for that thread, first
  std::unique_ptr<TopoRebuild> topo_async;
  // edges (topology; one list per differentiable-mesh set)
  DevBuf<int4> edges;   // v0, v1, vn0, vn1
  DevBuf<int2> edge_mi; // mesh, instance
  DevBuf<int2> edge_tris;  // the two flattened triangles sharing the edge (-1: boundary edge)
  int n_edges = 0;
  std::vector<int> edge_ids_key;  // dmesh ids the list was built for
  // views
  int n_views = 0, W = 0, H = 0;
  std::vector<CamDev> h_cams;
  DevBuf<CamDev> cams;
  DevBuf<float> ham;
  // per-call buffers
  DevBuf<float> images, targets, adj_in;
  DevBuf<int64_t> img_off;
  DevBuf<float4> adj;
  DevBuf<double> loss_part;
  DevBuf<double> loss_blk;        // chunk sums of the loss reduction
  DevBuf<unsigned> loss_ticket;   // its completion ticket (zeroed once)
  DevBuf<float> loss_out;  // 1 float: last loss
  DevBuf<float4> proj;     // per view per vertex projected position
  DevBuf<float> pmf, cdf;  // per view
  DevBuf<int4> queue;      // surviving edge samples
  DevBuf<int> queue_count;
  // the queue's shading order sorted by (view, edge) for coherent rays
  DevBuf<uint32_t> qkey[2], qhist;
  DevBuf<int> qidx[2], qn;
  // gradients
  std::vector<DLayout> dlay;
  std::vector<int> dmesh_ids;
  int64_t grad_total = 0;  // public gradient vector (DScene)
  int64_t grad_alloc = 0;  // + scratch matrix blocks of restricted meshes
  size_t grad_bytes() const { return sizeof(float) * (size_t)std::max<int64_t>(1, grad_alloc); }
  DevBuf<float> grad;
  DevBuf<uint32_t> err;
  OptState opt;
  // deterministic reduction (records, dense pairs, radix-sort scratch)
  int det = 0;
  // stored adjoint hits instead of re-tracing (one float4 per adjoint sample)
  int store_hits = 0;
  DevBuf<float4> hit_buf;
  DevBuf<uint32_t> rec_key, det_key[2], det_part, det_hist;
  DevBuf<float4> rec_val;
  DevBuf<int> rec_count, det_idx[2], det_n;
  DevBuf<DetFrag> det_frag;
  DevBuf<float> det_tr, det_tr_part;  // one transform block: dense per-sample values, block sums
  int det_tr_key = -1;                // its gradient index (-1: transform records instead)
  // work items
  std::vector<int4> h_pixel_items;
  int n_tiles_x = 0, n_tiles_y = 0;

  JobDev dev{};  // device view, refreshed by sync_dev()
};

// ---- launch helpers (implemented in the .cu files) --------------------------
void upload_scene(Job& J, const drgb_scene_desc* scene, cudaStream_t s);
void flatten_scene(Job& J, cudaStream_t s);            // instance transforms -> flattened arrays
void prepare_scene(Job& J, cudaStream_t s);            // flatten + traced triangles + refit
void commit_scene(Job& J, cudaStream_t s);             // flatten + LBVH build + refit
void rebuild_bvh(Job& J, cudaStream_t s);              // new topology from the current vertices + refit
void rebuild_bvh_begin(Job& J, cudaStream_t s);        // the same, overlapped with later steps...
void rebuild_bvh_poll(Job& J, cudaStream_t s);         // ...advanced between steps, never blocking
void rebuild_bvh_start(Job& J, cudaStream_t s);        // optimiser: built from this iteration's vertices...
void rebuild_bvh_apply(Job& J, cudaStream_t s);        // ...and used from a fixed later iteration on
void rebuild_bvh_discard(Job& J);                      // drop a rebuild in progress (waits for its thread)
void build_bvh(Job& J, cudaStream_t s);                // topology (Morton, sort, Karras)
void refit_bvh(Job& J, cudaStream_t s);
void setup_views(Job& J, const drgb_camera* cams, int n_views);
void sync_dev(Job& J);
void set_dscene(Job& J, const int32_t* ids, int n_ids, cudaStream_t s);
void build_edges(Job& J);
// Flattened block of instance 0 of a mesh (its instances' blocks follow).
int first_block(const Job& J, int mesh);
// The edge list of the meshes of `lay` (host vectors; build_edges uploads it).
void edge_list(const Job& J, const std::vector<DLayout>& lay, std::vector<int4>& ed, std::vector<int2>& mi,
               std::vector<int2>* tris = nullptr);
int64_t compute_layout(const Job& J, const int32_t* ids, int n_ids, std::vector<DLayout>& out,
                       int64_t* alloc_total = nullptr);
// TransformR::to_mat on the host (column-major, LiteMath's rounding).
void restricted_to_mat(const float* params7, float* out16);
// Restricted meshes: fold the scratch matrix gradient into the 7 parameters
// (after the gradient passes); rebuild the matrices from the parameters
// (after an optimiser step that changed them).
void launch_restricted_grad(Job& J, cudaStream_t s);
void launch_restricted_mats(Job& J, cudaStream_t s);
// The optimiser's view of one differentiable mesh.
OptMesh opt_mesh(const DLayout& L, MeshState& M);

void init_job_model(Job& J, int mode, int spp);
void choose_tile(int S, int& tw, int& th);
void camera_look_at(const float* o, const float* t, const float* u, float width, float height, float fov_rad,
                    float znear, float zfar, drgb_camera* out);
CamDev make_cam(const drgb_camera& c);

// Pixel kernel flags
// PX_HIT_STORE: adjoint pass that only traces and stores the primary hits;
// PX_HIT_LOAD: adjoint pass that reads them instead of tracing.
// PX_VIS: the raster pass of this call filled the job's visibility buffers
// (the pixel kernel reads them instead of tracing camera rays).
enum PixelFlags : int {
  PX_FWD = 1, PX_LOSS = 2, PX_ADJ = 4, PX_IMG = 8, PX_HIT_STORE = 16, PX_HIT_LOAD = 32, PX_VIS = 64
};
// Counters a buffer scanned by launch_rs_scan needs for m counters: the m
// counters (rounded up to 4) and one total per 16,384-counter tile.
inline size_t scan_scratch(size_t m) { return ((m + 3) & ~(size_t)3) + (m + 16383) / 16384; }
void launch_pixels(const JobDev* d_jobs, const int4* d_items, int n_items, int* d_counter, int flags, int grid,
                   cudaStream_t s, int mode, bool det = false);
void launch_loss_finalize(const JobDev* d_jobs, int n_jobs, cudaStream_t s);
// Rasterised primary visibility of the forward (passes & 1) and adjoint
// (passes & 2) samples of a single job's views, over ntx x nty tiles of
// tw x th pixels per view.
void launch_raster(const JobDev* d_job, const Job& J, int passes, int ntx, int nty, int tw, int th, cudaStream_t s);
// Raster tile of tw x th pixels for S samples per pixel.
void raster_tile(int S, int& tw, int& th);
// The size rule of the raster pass (without autotuning): at least 2 M
// forward camera samples per call, 64 triangles, and 32 forward samples per
// (view, triangle).
inline bool raster_pays(int64_t fwd_samples, int64_t n_views, int64_t n_tris) {
  return fwd_samples >= (2 << 20) && n_tris >= 64 && fwd_samples >= 32 * n_views * n_tris;
}
// Models whose raster records hold the shading point and u, v (JobDev::vis_uv_*).
inline bool vis_points(int mode) { return mode == LAMBERT_POINT_VCOLOR; }
// Light-space cells (G x G) of point-light shadow rays for the current geometry.
void launch_light_grid(const JobDev* d_job, const Job& J, int G, cudaStream_t s);
int light_grid_size(int n_tris);
void launch_rs_scan(uint32_t* hist, int m, cudaStream_t s);
void launch_adj_convert(const JobDev* d_job, int64_t n_pixels, cudaStream_t s);
void launch_cast(const JobDev* d_job, const CamDev* d_cam, const float* d_xy, int64_t n, uint32_t* prim,
                 uint32_t* inst, uint32_t* geom, float* t, float* u, float* v, cudaStream_t s);
void launch_edges(const JobDev* d_jobs, int job, const Job& J, int shade_grid, cudaStream_t s);
void launch_edges_prep(const JobDev* d_jobs, int job, int n_edges, int n_views, int n_vertices, cudaStream_t s);
void launch_edges_rest(const JobDev* d_jobs, int job, int n_edges, int n_views, int edge_samples, int* queue_count,
                       int shade_grid, cudaStream_t s, bool det, const Job* Jq, int mode);
// Blocks of the (atomic-scatter) pixel kernel of a model that one SM holds
// at a time (its register budget).
int pixel_blocks_resident(int mode);
void launch_opt_step(Job& J, cudaStream_t s);
void launch_opt_record(Job& J, cudaStream_t s);

// deterministic gradient reduction (detsum.cu)
void det_buffers(Job& J, cudaStream_t s);
void launch_det_clear(const Job& J, cudaStream_t s);
void launch_det_reduce(const Job& J, int sm_count, cudaStream_t s);
int sort_pairs_device(uint32_t* keys[2], int* vals[2], const int* n_ptr, int bits, uint32_t* hist, cudaStream_t s);
// Buffers of a batch's edge-queue sort (all null: shade in queue order).
struct QueueSort {
  uint32_t* keys[2];
  int* vals[2];
  uint32_t* hist;
  int* n;
  int bits;
};
constexpr int kSortGrid = 512;  // blocks of sort_pairs_device (its histogram has 256 * kSortGrid entries)

// edge random table shared by every job with the same sample count
const float* edge_random_table(int n, cudaStream_t s);
// The sample indices of that table ordered by their first number (the edge
// choice): selected in this order, consecutive samples fall on the same or
// neighbouring edges of the CDF.  Cached like the table.
const int* edge_random_order(int n, cudaStream_t s);
// The same 2n replayed random numbers in a host vector.
void edge_random_host(int n, std::vector<float>& out);

}  // namespace drgb
