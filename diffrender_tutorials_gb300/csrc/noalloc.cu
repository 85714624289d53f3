// drgb_d_render_and_compare_noalloc: forward + loss + interior adjoint + edge
// term without allocating GPU memory during the call.
//
// Who needs it: programs that hand out all device memory from a pool or
// budget of their own and forbid allocations once they run -- an engine or
// a server that sizes its HBM at start-up and treats a later cudaMalloc as
// an error -- and loops that must not pay for an allocation, nor for the
// device-wide synchronisation that cudaMalloc and cudaFree can cause, in
// the middle of a run.  drgb_d_render_and_compare_device grows its per-call
// buffers with cudaMalloc on first use; this variant takes every per-call
// buffer from one fixed array compiled into the library instead.
//
// Limits and sharing:
//  * the array holds kScratchBytes (32 MiB).  A call whose buffers (adjoint
//    images, edge-sample queue, tile partials, projected vertices, edge
//    sampler, random streams) need more is rejected with DRGB_ERR_INVALID;
//    roughly one 512x512 view with 262,144 edge samples fits;
//  * the first call on a device looks the array's device address up with
//    cudaGetSymbolAddress (the CUDA runtime may load the array onto that
//    device only then); make that first call before any stream capture.
//    From then on the array stays on the device until the process exits;
//  * all calls share the one array and it keeps the previous call's
//    contents: each call clears what must start at zero (the caller's
//    gradient vector, the sample-queue and work-queue counters) and rewrites
//    the rest, so calls that overlap on the GPU -- from two host threads, or
//    enqueued on different streams without ordering -- race on it;
//  * host cost per call: the edge list (a sort of 3 x triangles entries) and
//    the 2 x edge_samples replayed random numbers are rebuilt on the host and
//    copied from pageable memory, and the call waits for its stream at the
//    end to read the kernels' error flag.
// The renderer itself (scene, hierarchy, model constants) must have been
// committed beforehand; that set-up allocates as usual.
#include <mutex>

#include "renderer.h"

namespace drgb {

void launch_edges_raw(const JobDev* d_jobs, int job, int n_edges, int n_views, int n_vertices, int edge_samples,
                      int* queue_count, int shade_grid, cudaStream_t s, bool det, const Job* Jq, int mode);

constexpr size_t kScratchBytes = 32u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

// Device address of the scratch array, looked up once per device.
unsigned char* scratch_address(int device) {
  static std::mutex mu;
  static std::vector<unsigned char*> addr;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)addr.size() <= device) addr.resize(device + 1, nullptr);
  if (!addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      throw CudaError(std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e), DRGB_ERR_CUDA);
    addr[device] = static_cast<unsigned char*>(p);
  }
  return addr[device];
}

// Bump allocator over the scratch array (256-byte aligned regions).
struct Carve {
  size_t used = 0;
  template <class T>
  size_t take(size_t count) {
    const size_t off = (used + 255) & ~size_t(255);
    used = off + count * sizeof(T);
    return off;
  }
};

}  // namespace
}  // namespace drgb

extern "C" int drgb_d_render_and_compare_noalloc(drgb_renderer* r, const drgb_camera* cams, const float* d_targets,
                                                 int n_views, int edge_samples, const int32_t* ids, int n_ids,
                                                 float* d_dscene, float* d_loss) {
  return guard([&] {
    require(r != nullptr, "null renderer");
    r->require_commit();
    require(cams && d_targets && d_dscene && d_loss && n_views > 0, "null argument");
    require(edge_samples >= 0, "edge sample count must be >= 0");
    require(!r->job.det, "deterministic mode needs its record buffers; use drgb_d_render_and_compare_device",
            DRGB_ERR_UNSUPPORTED);
    for (int i = 1; i < n_views; i++)
      require((int)cams[i].width == (int)cams[0].width && (int)cams[i].height == (int)cams[0].height,
              "gradient calls need all views of the same size");
    r->set_device();
    Job& J = r->job;
    unsigned char* base = scratch_address(r->device);

    // ---- host-side description of the call (no device memory involved) ----
    const int W = (int)cams[0].width, H = (int)cams[0].height;
    require(W >= 1 && H >= 1, "camera size must be positive");
    std::vector<CamDev> hc(n_views);
    for (int i = 0; i < n_views; i++) hc[i] = make_cam(cams[i]);
    std::vector<int64_t> off(n_views + 1, 0);
    for (int i = 0; i < n_views; i++) off[i + 1] = off[i] + (int64_t)W * H;
    std::vector<int4> items;
    for (int v = 0; v < n_views; v++)
      for (int y = 0; y < H; y += J.tile_h)
        for (int x = 0; x < W; x += J.tile_w) items.push_back(make_int4(0, v, x, y));
    std::vector<DLayout> lay;
    const int64_t grad_total = compute_layout(J, ids, n_ids, lay);
    for (const DLayout& L : lay)
      require(L.rt_off < 0, "restricted-transform meshes need drgb_d_render_and_compare_device (the Jacobian step "
                            "works on a scratch block the caller's gradient vector has no room for)");
    std::vector<MeshDev> md(J.meshes.size());
    for (size_t m = 0; m < J.meshes.size(); m++) {
      const MeshState& M = J.meshes[m];
      md[m] = MeshDev{M.texture.p, M.tex_w, M.tex_h, M.tex_c, -1, 0, 0, -1, -1, 0, M.nv, M.n_inst, first_block(J, (int)m)};
    }
    for (size_t k = 0; k < lay.size(); k++) {
      MeshDev& d = md[lay[k].mesh_id];
      d.dslot = (int)k;
      d.g_base = lay[k].base;
      d.pos_off = lay[k].pos_off;
      d.color_off = lay[k].color_off;
      d.tex_off = lay[k].tex_off;
      d.tr_off = lay[k].tr_off;
    }
    std::vector<int4> ed;
    std::vector<int2> emi, etris;
    edge_list(J, lay, ed, emi, &etris);
    const int E = (int)ed.size();
    std::vector<float> rnd;
    if (edge_samples > 0) edge_random_host(edge_samples, rnd);

    // ---- carve the scratch array ----
    Carve c;
    const size_t o_job = c.take<JobDev>(1);
    const size_t o_cams = c.take<CamDev>(n_views);
    const size_t o_off = c.take<int64_t>(n_views + 1);
    const size_t o_items = c.take<int4>(items.size());
    const size_t o_part = c.take<double>(items.size());
    const size_t o_md = c.take<MeshDev>(std::max<size_t>(1, md.size()));
    const size_t o_adj = c.take<float4>((size_t)n_views * W * H);
    const size_t o_proj = c.take<float4>((size_t)n_views * std::max(1, J.n_vertices));
    const size_t o_pmf = c.take<float>((size_t)n_views * std::max(1, E));
    const size_t o_cdf = c.take<float>((size_t)n_views * (E + 1));
    const size_t o_queue = c.take<int4>((size_t)n_views * std::max(1, edge_samples));
    const size_t o_edges = c.take<int4>(std::max(1, E));
    const size_t o_emi = c.take<int2>(std::max(1, E));
    const size_t o_etri = c.take<int2>(std::max(1, E));
    const size_t o_rnd = c.take<float>(std::max<size_t>(1, rnd.size()));
    const size_t o_lblk = c.take<double>((size_t)n_views * kLossBlocks);
    const size_t o_cnt = c.take<int>(4);
    if (c.used > kScratchBytes)
      throw CudaError("drgb_d_render_and_compare_noalloc: this call needs " + std::to_string(c.used) +
                          " bytes of scratch; the fixed array holds " + std::to_string(kScratchBytes) +
                          " bytes (use drgb_d_render_and_compare_device for larger calls)",
                      DRGB_ERR_INVALID);

    // ---- device view of the job: scene from the committed renderer, every
    // per-call buffer inside the scratch array, inputs/outputs from the caller
    JobDev d{};
    d.n_vertices = J.n_vertices;
    d.n_tris = J.n_tris;
    d.n_blocks = J.n_blocks;
    d.n_meshes = (int)J.meshes.size();
    d.pos = J.pos.p;
    d.orig = J.orig.p;
    d.col = J.col.p;
    d.nrm = J.nrm.p;
    d.tan = J.tan.p;
    d.tc = J.tc.p;
    d.tri_v = J.tri_v.p;
    d.blocks = J.blocks.p;
    d.meshes = reinterpret_cast<const MeshDev*>(base + o_md);
    d.tr_inv0 = J.tr_inv0.p;
    d.block_tr = J.block_tr.p;
    d.nodes = J.nodes.p;
    d.nodes4 = J.nodes4.p;
    d.tri = J.tri.p;
    d.leaf_of = J.leaf_of.p;
    d.root = J.root;
    d.trace_bruteforce = J.trace_bruteforce;
    d.trace_limit = J.trace_limit;
    d.edge_exact = J.edge_exact;
    d.mode = J.mode;
    d.spp = J.spp;
    d.sq = J.sq;
    d.S = J.S;
    d.ham = J.ham.p;
    d.mp = J.mp;
    d.n_views = n_views;
    d.cams = reinterpret_cast<const CamDev*>(base + o_cams);
    d.W = W;
    d.H = H;
    d.grad = d_dscene;
    d.err = J.err.p;
    d.images = nullptr;
    d.img_off = reinterpret_cast<const int64_t*>(base + o_off);
    d.targets = d_targets;
    d.adj = reinterpret_cast<float4*>(base + o_adj);
    d.adj_in = nullptr;
    d.loss_part = reinterpret_cast<double*>(base + o_part);
    d.loss_blk = reinterpret_cast<double*>(base + o_lblk);
    d.loss_out = d_loss;
    d.tile_w = J.tile_w;
    d.tile_h = J.tile_h;
    d.item_base = 0;
    d.item_count = (int)items.size();
    d.edges = reinterpret_cast<const int4*>(base + o_edges);
    d.edge_mi = reinterpret_cast<const int2*>(base + o_emi);
    d.edge_tris = reinterpret_cast<const int2*>(base + o_etri);
    d.edge_sil = J.edge_sil;
    d.n_edges = E;
    d.proj = reinterpret_cast<float4*>(base + o_proj);
    d.pmf = reinterpret_cast<float*>(base + o_pmf);
    d.cdf = reinterpret_cast<float*>(base + o_cdf);
    d.queue = reinterpret_cast<int4*>(base + o_queue);
    // [0] edge-sample queue, [1] its shading counter, [2] pixel work queue, [3] loss ticket
    int* counters = reinterpret_cast<int*>(base + o_cnt);
    d.queue_count = counters;
    d.loss_ticket = reinterpret_cast<unsigned*>(counters + 3);
    d.queue_cap = n_views * std::max(1, edge_samples);
    d.edge_samples = edge_samples;
    d.rnd = reinterpret_cast<const float*>(base + o_rnd);
    d.work = nullptr;

    // ---- copies into the scratch array (pageable host sources; the copies
    // complete their host reads before returning) and the launches ----
    cudaStream_t s = r->stream;
    auto put = [&](size_t o, const void* src, size_t bytes) {
      if (bytes) DRGB_CUDA(cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, s));
    };
    put(o_job, &d, sizeof(JobDev));
    put(o_cams, hc.data(), sizeof(CamDev) * hc.size());
    put(o_off, off.data(), sizeof(int64_t) * off.size());
    put(o_items, items.data(), sizeof(int4) * items.size());
    put(o_md, md.data(), sizeof(MeshDev) * md.size());
    put(o_edges, ed.data(), sizeof(int4) * ed.size());
    put(o_emi, emi.data(), sizeof(int2) * emi.size());
    put(o_etri, etris.data(), sizeof(int2) * etris.size());
    if (edge_samples > 0) put(o_rnd, rnd.data(), sizeof(float) * rnd.size());
    if (grad_total > 0) DRGB_CUDA(cudaMemsetAsync(d_dscene, 0, sizeof(float) * grad_total, s));
    DRGB_CUDA(cudaMemsetAsync(counters, 0, 4 * sizeof(int), s));
    const JobDev* d_job = reinterpret_cast<const JobDev*>(base + o_job);
    const int flags = PX_FWD | PX_LOSS | (J.mode != SILHOUETTE ? PX_ADJ : 0);
    launch_pixels(d_job, reinterpret_cast<const int4*>(base + o_items), (int)items.size(), counters + 2, flags,
                  r->px_grid(), s, J.mode);
    launch_loss_finalize(d_job, 1, s);
    if (edge_samples > 0)
      launch_edges_raw(d_job, 0, E, n_views, J.n_vertices, edge_samples, counters, r->edge_grid(), s, false, nullptr,
                       J.mode);
    uint32_t f = 0;
    DRGB_CUDA(cudaMemcpyAsync(&f, J.err.p, sizeof(f), cudaMemcpyDeviceToHost, s));
    DRGB_CUDA(cudaStreamSynchronize(s));
    if (f) {
      DRGB_CUDA(cudaMemsetAsync(J.err.p, 0, sizeof(uint32_t), s));
      DRGB_CUDA(cudaStreamSynchronize(s));
      throw CudaError("kernel error flags " + std::to_string(f), DRGB_ERR_KERNEL);
    }
  });
}
