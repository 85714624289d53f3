// GPU IDiffRender / IOptimizer over the drgb C ABI.  See gpu_drender.h.
//
// Reference interfaces implemented (file:line in FROL256/diffrender_tutorials):
//   IDiffRender            src/virtual_drender.h:14-26
//   DiffRender semantics   src/drender.h:91-191 (commit, render, d_render,
//                          d_render_and_compare)
//   IOptimizer / OptSimple src/optimizer.h:52-61, src/optimizer_simple.cpp:272-309
// Data passed through unchanged: LiteMath float3 / float2 arrays are packed
// floats, float4x4 is column major -- the layouts drgb.h expects.
#include "gpu_drender.h"

#include <cstdio>
#include <cstring>
#include <vector>

#include "drgb.h"

namespace diff_render {
namespace {

thread_local int t_code = 0;
thread_local std::string t_msg;

bool ok(int rc, const char* where) {
  t_code = rc;
  if (rc == DRGB_OK) {
    t_msg.clear();
    return true;
  }
  char buf[512];
  drgb_last_error(buf, sizeof(buf));
  t_msg = buf;
  std::printf("[%s]: error %d: %s\n", where, rc, buf);
  return false;
}

// drgb_scene_desc over a Scene's arrays (kept alive by this object).
struct SceneView {
  std::vector<drgb_mesh_desc> meshes;
  std::vector<std::vector<float>> rparams;  // TransformR parameters, 7 per instance
  drgb_scene_desc desc{};

  explicit SceneView(const Scene& s) {
    const auto& ms = s.get_meshes();
    meshes.resize(ms.size());
    rparams.resize(ms.size());
    for (size_t i = 0; i < ms.size(); i++) {
      const TriangleMesh& m = ms[i];
      drgb_mesh_desc& d = meshes[i];
      std::memset(&d, 0, sizeof(d));
      d.n_vertices = (int32_t)m.vertices.size();
      d.n_indices = (int32_t)m.indices.size();
      d.vertices = reinterpret_cast<const float*>(m.vertices.data());
      d.colors = m.colors.empty() ? nullptr : reinterpret_cast<const float*>(m.colors.data());
      d.tc = m.tc.empty() ? nullptr : reinterpret_cast<const float*>(m.tc.data());
      d.normals = m.normals.empty() ? nullptr : reinterpret_cast<const float*>(m.normals.data());
      d.tangents = m.tangents.empty() ? nullptr : reinterpret_cast<const float*>(m.tangents.data());
      d.indices = m.indices.data();
      if (s.get_instancing_type((unsigned)i) == Scene::RESTRICTED_TRANSFORM) {
        for (const TransformR& r : s.get_restricted_transform((unsigned)i)) {
          const float p[7] = {r.translate.x, r.translate.y, r.translate.z, r.rotate.x, r.rotate.y, r.rotate.z,
                              r.scale};
          rparams[i].insert(rparams[i].end(), p, p + 7);
        }
        d.n_instances = (int32_t)(rparams[i].size() / 7);
        d.restricted = rparams[i].empty() ? nullptr : rparams[i].data();
      } else {
        const std::vector<float4x4>& tr = s.get_transform((unsigned)i);
        d.n_instances = (int32_t)tr.size();
        d.transforms = tr.empty() ? nullptr : reinterpret_cast<const float*>(tr.data());
      }
      if (!m.textures.empty()) {
        const CPUTexture& t = m.textures[0];
        d.tex_w = t.w;
        d.tex_h = t.h;
        d.tex_channels = t.channels;
        d.texture = t.data();
      }
    }
    desc.n_meshes = (int32_t)meshes.size();
    desc.meshes = meshes.data();
  }
};

std::vector<drgb_camera> cameras(const CamInfo* cams, int n) {
  std::vector<drgb_camera> out((size_t)n);
  for (int i = 0; i < n; i++) {
    std::memcpy(out[i].world_view, &cams[i].mWorldView, 16 * sizeof(float));
    std::memcpy(out[i].proj, &cams[i].mProj, 16 * sizeof(float));
    out[i].width = cams[i].width;
    out[i].height = cams[i].height;
  }
  return out;
}

std::vector<int32_t> dmesh_ids(DScene& ds) {
  std::vector<int32_t> ids;
  for (DMesh& m : ds.get_dmeshes()) ids.push_back(m.get_mesh_id());
  return ids;
}

// The gradient blocks of a DScene, concatenated in dmesh order (the layout
// of drgb_dscene_layout), and back.
std::vector<float> gather(DScene& ds) {
  std::vector<float> v;
  for (DMesh& m : ds.get_dmeshes()) v.insert(v.end(), m.full_data(), m.full_data() + m.full_size());
  return v;
}
void scatter(const std::vector<float>& v, DScene& ds) {
  size_t off = 0;
  for (DMesh& m : ds.get_dmeshes()) {
    std::memcpy(m.full_data(), v.data() + off, sizeof(float) * m.full_size());
    off += m.full_size();
  }
}

// The gradient vector drgb fills must have the DScene's size.
bool layout_matches(drgb_renderer* r, const std::vector<int32_t>& ids, DScene& ds, const char* where) {
  int64_t total = 0;
  std::vector<int32_t> lay(9 * ids.size() + 9);
  if (!ok(drgb_dscene_layout(r, ids.data(), (int)ids.size(), lay.data(), &total), where)) return false;
  if (total != (int64_t)ds.full_size()) {
    t_code = DRGB_ERR_UNSUPPORTED;
    t_msg = "gradient layout differs from the DScene";
    std::printf("[%s]: error, %s\n", where, t_msg.c_str());
    return false;
  }
  return true;
}

class GpuDiffRender : public IDiffRender {
 public:
  explicit GpuDiffRender(int device) : device_(device) {}
  ~GpuDiffRender() override {
    if (r_) drgb_renderer_destroy(r_);
  }

  void init(const DiffRenderSettings& s) override {
    mode = s.mode;
    if (r_) {
      drgb_renderer_destroy(r_);
      r_ = nullptr;
    }
    ok(drgb_renderer_create((int)s.mode, s.spp, device_, &r_), "GpuDiffRender::init");
  }

  void commit(const Scene& scene) override {
    if (!r_) return;
    SceneView sv(scene);
    if (ok(drgb_commit(r_, &sv.desc), "GpuDiffRender::commit")) last_ = &scene;
  }

  void render(const Scene& scene, const CamInfo* cams, Img* images, int n) override {
    if (!ready(scene, "GpuDiffRender::render")) return;
    auto c = cameras(cams, n);
    size_t total = 0;
    for (int i = 0; i < n; i++) total += (size_t)cams[i].width * (size_t)cams[i].height;
    std::vector<float> buf(3 * total);
    if (!ok(drgb_render(r_, c.data(), n, buf.data()), "GpuDiffRender::render")) return;
    size_t off = 0;
    for (int i = 0; i < n; i++) {
      const size_t px = (size_t)cams[i].width * (size_t)cams[i].height;
      if ((size_t)images[i].width() * images[i].height() == px)
        std::memcpy(images[i].data(), buf.data() + 3 * off, sizeof(float) * 3 * px);
      off += px;
    }
  }

  void d_render(const Scene& scene, const CamInfo* cams, const Img* adjoints, int n, const int edge_samples,
                DScene& d_mesh, Img* debug = nullptr, int n_debug = 0) override {
    (void)debug;
    (void)n_debug;
    if (!ready(scene, "GpuDiffRender::d_render")) return;
    auto c = cameras(cams, n);
    std::vector<float> adj;
    for (int i = 0; i < n; i++) {
      const float* p = reinterpret_cast<const float*>(adjoints[i].data());
      adj.insert(adj.end(), p, p + 3 * (size_t)adjoints[i].width() * adjoints[i].height());
    }
    auto ids = dmesh_ids(d_mesh);
    if (!layout_matches(r_, ids, d_mesh, "GpuDiffRender::d_render")) return;
    auto g = gather(d_mesh);
    if (ok(drgb_d_render(r_, c.data(), adj.data(), n, edge_samples, ids.data(), (int)ids.size(), g.data()),
           "GpuDiffRender::d_render"))
      scatter(g, d_mesh);
  }

  float d_render_and_compare(const Scene& scene, const CamInfo* cams, const Img* targets, int n,
                             const int edge_samples, DScene& d_mesh, Img* out_images = nullptr) override {
    if (!r_) return 0.0f;
    commit(scene);  // as the reference does (src/drender.h:176)
    if (last_ != &scene) return 0.0f;
    auto c = cameras(cams, n);
    std::vector<float> tg;
    for (int i = 0; i < n; i++) {
      const float* p = reinterpret_cast<const float*>(targets[i].data());
      tg.insert(tg.end(), p, p + 3 * (size_t)targets[i].width() * targets[i].height());
    }
    auto ids = dmesh_ids(d_mesh);
    if (!layout_matches(r_, ids, d_mesh, "GpuDiffRender::d_render_and_compare")) return 0.0f;
    std::vector<float> g((size_t)d_mesh.full_size(), 0.0f);
    std::vector<float> imgs;
    if (out_images) imgs.resize(3 * (size_t)n * (size_t)cams[0].width * (size_t)cams[0].height);
    float loss = 0.0f;
    if (!ok(drgb_d_render_and_compare(r_, c.data(), tg.data(), n, edge_samples, ids.data(), (int)ids.size(),
                                      g.data(), out_images ? imgs.data() : nullptr, &loss),
            "GpuDiffRender::d_render_and_compare"))
      return 0.0f;
    scatter(g, d_mesh);
    if (out_images) {
      const size_t px = (size_t)cams[0].width * (size_t)cams[0].height;
      for (int i = 0; i < n; i++) {
        out_images[i].resize((unsigned)cams[i].width, (unsigned)cams[i].height);
        std::memcpy(out_images[i].data(), imgs.data() + 3 * px * i, sizeof(float) * 3 * px);
      }
    }
    return loss;
  }

  drgb_renderer* handle() const { return r_; }
  int device() const { return device_; }

 private:
  bool ready(const Scene& scene, const char* where) {
    if (!r_) return false;
    if (&scene != last_) {
      std::printf("[%s]: error, renderer was not prepared for this scene!\n", where);
      return false;
    }
    return true;
  }

  int device_;
  drgb_renderer* r_ = nullptr;
  const Scene* last_ = nullptr;
};

class GpuOptimizer : public IOptimizer {
 public:
  explicit GpuOptimizer(int device) : device_(device) {}
  ~GpuOptimizer() override {
    if (own_ && r_) drgb_renderer_destroy(r_);
  }

  void Init(const Scene& scene, std::shared_ptr<IDiffRender> dr, const CamInfo* cams, const Img* targets, int n,
            OptimizerParameters p) override {
    scene_ = scene;
    params_ = p;
    // the GPU renderer's own state when it is one, else a renderer of the same model
    auto* g = dynamic_cast<GpuDiffRender*>(dr.get());
    if (own_ && r_) drgb_renderer_destroy(r_);
    r_ = nullptr;
    own_ = false;
    holder_ = dr;
    if (g && g->handle()) {
      r_ = g->handle();
    } else {
      // a fresh renderer with the model; spp is not part of IDiffRender, so the
      // reference default of the tests (16) is used
      if (!ok(drgb_renderer_create((int)dr->mode, 16, device_, &r_), "GpuOptimizer::Init")) return;
      own_ = true;
    }
    drgb_opt_params op;
    std::memset(&op, 0, sizeof(op));
    op.alg = (int32_t)p.alg;
    op.decay_period = p.decayPeriod;
    op.decay_mult = p.decay_mult;
    op.base_lr = p.base_lr;
    op.position_lr = p.position_lr;
    op.textures_lr = p.textures_lr;
    op.transforms_lr = p.transforms_lr;
    op.flags = p.flags;
    op.n_dmesh_ids = (int32_t)p.differentiable_mesh_ids.size();
    for (int i = 0; i < op.n_dmesh_ids && i < 16; i++) op.dmesh_ids[i] = p.differentiable_mesh_ids[i];
    auto c = cameras(cams, n);
    std::vector<float> tg;
    for (int i = 0; i < n; i++) {
      const float* q = reinterpret_cast<const float*>(targets[i].data());
      tg.insert(tg.end(), q, q + 3 * (size_t)targets[i].width() * targets[i].height());
    }
    SceneView sv(scene_);
    ready_ = ok(drgb_optimizer_init(r_, &sv.desc, c.data(), tg.data(), n, &op), "GpuOptimizer::Init");
  }

  Scene Run(size_t iters, float& final_error, std::vector<Scene>* dump = nullptr) override {
    final_error = 0.0f;
    if (!ready_) return scene_;
    if (dump) {
      for (size_t i = 0; i < iters; i++) {
        if (!ok(drgb_optimizer_run(r_, 1, &final_error, nullptr), "GpuOptimizer::Run")) break;
        fetch();
        dump->push_back(scene_);
      }
    } else {
      if (ok(drgb_optimizer_run(r_, (int64_t)iters, &final_error, nullptr), "GpuOptimizer::Run")) fetch();
    }
    if (params_.verbose) std::printf("GpuOptimizer: %zu iterations, final MSE %g\n", iters, final_error);
    return scene_;
  }

 private:
  // The optimised meshes back into the host scene.
  void fetch() {
    auto& meshes = scene_.get_meshes_modify();
    for (size_t i = 0; i < meshes.size(); i++) {
      TriangleMesh& m = meshes[i];
      std::vector<float4x4> tr = scene_.get_transform((unsigned)i);
      float* tex = m.textures.empty() ? nullptr : m.textures[0].data();
      const bool own_tr = scene_.get_instancing_type((unsigned)i) != Scene::RESTRICTED_TRANSFORM && !tr.empty();
      ok(drgb_optimizer_get_mesh(r_, (int)i, reinterpret_cast<float*>(m.vertices.data()),
                                 m.colors.empty() ? nullptr : reinterpret_cast<float*>(m.colors.data()), tex,
                                 own_tr ? reinterpret_cast<float*>(tr.data()) : nullptr),
         "GpuOptimizer::Run");
      if (own_tr) scene_.get_transform_modify((unsigned)i) = tr;
      if (scene_.get_instancing_type((unsigned)i) == Scene::RESTRICTED_TRANSFORM) {
        auto& rts = scene_.get_restricted_transform_modify((unsigned)i);
        std::vector<float> p(7 * rts.size());
        if (p.empty() || !ok(drgb_optimizer_get_restricted(r_, (int)i, p.data()), "GpuOptimizer::Run")) continue;
        for (size_t j = 0; j < rts.size(); j++) {
          const float* q = &p[7 * j];
          rts[j].translate = float3(q[0], q[1], q[2]);
          rts[j].rotate = float3(q[3], q[4], q[5]);
          rts[j].scale = q[6];
        }
      }
    }
  }

  int device_;
  drgb_renderer* r_ = nullptr;
  bool own_ = false;
  bool ready_ = false;
  std::shared_ptr<IDiffRender> holder_;
  Scene scene_;
  OptimizerParameters params_;
};

}  // namespace

std::shared_ptr<IDiffRender> MakeGpuDifferentialRenderer(const DiffRenderSettings& settings, int device) {
  auto r = std::make_shared<GpuDiffRender>(device);
  r->init(settings);
  return r;
}

std::shared_ptr<IOptimizer> CreateGpuOptimizer(int device) { return std::make_shared<GpuOptimizer>(device); }

int last_error(std::string* message) {
  if (message) *message = t_msg;
  return t_code;
}

}  // namespace diff_render
