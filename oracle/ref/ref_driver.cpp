// Driver that runs the reference renderer's own CPU code (brute-force caster,
// OpenMP) on scenes described in a DRKV file and dumps its outputs, so that
// golden fixtures and the oracle restatement can be pinned to the reference.
// Test infrastructure only: it links the reference sources compiled by
// oracle/ref/build_ref.py and is never part of the product path.
//
// Public reference API used (file:line in the reference project):
//   MakeDifferentialRenderer          src/drender.cpp:89-147
//   IDiffRender::{commit,render,d_render,d_render_and_compare}
//                                     src/virtual_drender.h:14-26
//   MakeRayTracer3D / CastSingleRay   raytrace_src/raytrace3d_bf.cpp:158-189
//   CreateSimpleOptimizer / Run       src/optimizer.h:52-61, src/optimizer_simple.cpp:272-309
//   CamInfo                           common_src/camera.h:6-44
//   qmc::planeHammersley, prng::*     common_src/qmc.cpp:227-268
//   mesh_utils::LoadMeshFromVSGF      common_src/cmesh.cpp:139-170
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "drender.h"
#include "optimizer.h"
#include "qmc.h"
#include "cmesh.h"
#include "raytrace.h"
#include "kvio.h"
#include "ref_pointlight.h"
#include "scenes.h"
#include "oracle.h"
#ifdef DRGB_WITH_GPU
#include "gpu_drender.h"  // the GPU IDiffRender / IOptimizer (diffrender_tutorials_gb300/cpp)
#endif

using namespace diff_render;

// The Enzyme plugin is absent, so the restricted-transform Jacobian it
// would produce (src/drender_autodiff.cpp:97-107, the forward derivative of
// dmat_dtransforms_jac_f, :78-95) comes from the oracle's analytic form of
// the same derivative (oracle.c, orc_restricted_jacobian; pinned against
// central differences of to_mat by the tests).  Everything around it -- the
// chain rule over the 12 matrix gradients, the layout, the optimiser update
// -- is the reference's own code.  `mat` is TransformR::M, which to_mat()
// fills in the patched scene.h (build_ref.py).
void dmat_dtransforms_jac(float const mat[7], float jac[7][12]) { orc_restricted_jacobian(mat, &jac[0][0]); }

// backend 0: the reference's CPU renderer; 1: the GPU renderer behind the
// same interface (the reference's own code drives it); 2 (optimiser task):
// the GPU optimiser as well.
// Mode 16 (point light, vertex albedo) runs the reference's DiffRender<>
// with the model of ref_pointlight.h (instantiated in drender_unit.cpp); its
// gradients use the VERTEX_COLOR layout, which IDiffRender::mode reports so
// that OptSimple allocates it.
namespace diff_render {
std::shared_ptr<IDiffRender> MakePointLightRenderer(const DiffRenderSettings& settings);
}
static std::shared_ptr<IDiffRender> make_renderer(const kv::File& in, SHADING_MODEL mode, int spp) {
#ifdef DRGB_WITH_GPU
  if (in.i("backend", 0) >= 1) return MakeGpuDifferentialRenderer(DiffRenderSettings{mode, spp});
#endif
  if (mode == kPointLightVColor) return MakePointLightRenderer(DiffRenderSettings{mode, spp});
  return MakeDifferentialRenderer(DiffRenderSettings{mode, spp});
}

static SHADING_MODEL layout_mode(SHADING_MODEL m) {
  return m == kPointLightVColor ? SHADING_MODEL::VERTEX_COLOR : m;
}

static std::string key(int m, const char* what) { return "m" + std::to_string(m) + "." + what; }

static void build_scene(const kv::File& in, Scene& scene) {
  const int n_meshes = in.i("n_meshes");
  for (int m = 0; m < n_meshes; m++) {
    TriangleMesh mesh;
    auto v = in.vec<float>(key(m, "vertices"));
    for (size_t k = 0; k < v.size() / 3; k++) mesh.vertices.push_back(float3(v[3 * k], v[3 * k + 1], v[3 * k + 2]));
    if (in.has(key(m, "colors"))) {
      auto c = in.vec<float>(key(m, "colors"));
      for (size_t k = 0; k < c.size() / 3; k++) mesh.colors.push_back(float3(c[3 * k], c[3 * k + 1], c[3 * k + 2]));
    }
    if (in.has(key(m, "tc"))) {
      auto c = in.vec<float>(key(m, "tc"));
      for (size_t k = 0; k < c.size() / 2; k++) mesh.tc.push_back(float2(c[2 * k], c[2 * k + 1]));
    }
    if (in.has(key(m, "normals"))) {
      auto c = in.vec<float>(key(m, "normals"));
      for (size_t k = 0; k < c.size() / 3; k++) mesh.normals.push_back(float3(c[3 * k], c[3 * k + 1], c[3 * k + 2]));
    }
    if (in.has(key(m, "tangents"))) {
      auto c = in.vec<float>(key(m, "tangents"));
      for (size_t k = 0; k < c.size() / 3; k++) mesh.tangents.push_back(float3(c[3 * k], c[3 * k + 1], c[3 * k + 2]));
    }
    mesh.indices = in.vec<uint32_t>(key(m, "indices"));
    if (in.has(key(m, "tex"))) {
      auto shape = in.vec<int32_t>(key(m, "tex_shape"));
      CPUTexture t;
      t.w = shape[0];
      t.h = shape[1];
      t.channels = shape[2];
      t.m_data = in.vec<float>(key(m, "tex"));
      mesh.textures.push_back(t);
    }
    if (in.has(key(m, "restricted"))) {  // Scene::add_mesh with TransformR (scene.h:140-148)
      auto rp = in.vec<float>(key(m, "restricted"));
      std::vector<TransformR> rts;
      for (size_t k = 0; k < rp.size() / 7; k++) {
        const float* q = rp.data() + 7 * k;
        rts.push_back(TransformR(float3(q[0], q[1], q[2]), float3(q[3], q[4], q[5]), q[6]));
      }
      scene.add_mesh(mesh, rts);
      continue;
    }
    std::vector<float4x4> trs;
    if (in.has(key(m, "transforms"))) {
      auto tv = in.vec<float>(key(m, "transforms"));
      for (size_t k = 0; k < tv.size() / 16; k++) {
        float4x4 M;
        std::memcpy((void*)&M, tv.data() + 16 * k, 16 * sizeof(float));  // LiteMath memory = column major
        trs.push_back(M);
      }
    } else {
      trs.push_back(float4x4());
    }
    scene.add_mesh(mesh, trs);
  }
}

static std::vector<CamInfo> build_cams(const kv::File& in) {
  std::vector<CamInfo> cams;
  if (in.has("cams_lookat")) {
    auto c = in.vec<float>("cams_lookat");
    std::vector<float> fov = in.has("cams_fov") ? in.vec<float>("cams_fov") : std::vector<float>();
    int n = (int)(c.size() / 11);
    for (int i = 0; i < n; i++) {
      const float* p = c.data() + 11 * i;
      float f = fov.empty() ? (float)M_PI_4 : fov[i];
      cams.push_back(CamInfo(float3(p[0], p[1], p[2]), float3(p[3], p[4], p[5]), float3(p[6], p[7], p[8]), p[9], p[10], f));
    }
  } else {
    auto c = in.vec<float>("cams_mat");
    int n = (int)(c.size() / 34);
    for (int i = 0; i < n; i++) {
      const float* p = c.data() + 34 * i;
      CamInfo cam;
      std::memcpy((void*)&cam.mWorldView, p, 16 * sizeof(float));
      std::memcpy((void*)&cam.mProj, p + 16, 16 * sizeof(float));
      cam.width = p[32];
      cam.height = p[33];
      cam.commit();
      cams.push_back(cam);
    }
  }
  return cams;
}

static std::vector<float> mat_to_vec(const float4x4& m) {
  std::vector<float> v(16);
  std::memcpy(v.data(), (const void*)&m, 16 * sizeof(float));
  return v;
}

static void images_in(const kv::File& in, const char* name, const std::vector<CamInfo>& cams, std::vector<Img>& imgs) {
  auto data = in.vec<float>(name);
  imgs.resize(cams.size());
  size_t off = 0;
  for (size_t i = 0; i < cams.size(); i++) {
    int w = (int)cams[i].width, h = (int)cams[i].height;
    imgs[i].resize(w, h);
    std::memcpy((void*)imgs[i].data(), data.data() + off, sizeof(float) * 3 * w * h);
    off += 3 * (size_t)w * h;
  }
}

static void images_out(kv::File& out, const char* name, const std::vector<Img>& imgs) {
  std::vector<float> all;
  for (auto& im : imgs) {
    const float* p = (const float*)im.data();
    all.insert(all.end(), p, p + 3 * im.width() * im.height());
  }
  out.put_f32(name, all);
}

static void dscene_out(kv::File& out, DScene& ds) {
  int k = 0;
  for (auto& dm : ds.get_dmeshes()) {
    std::string base = "dmesh" + std::to_string(k);
    std::vector<float> data(dm.full_data(), dm.full_data() + dm.full_size());
    out.put_f32(base, data);
    GradReal* p0 = dm.full_data();
    std::vector<int32_t> layout = {dm.vertex_count(), dm.instance_count(),
                                   dm.pos(0) ? (int)(dm.pos(0) - p0) : -1,
                                   dm.color(0) ? (int)(dm.color(0) - p0) : -1,
                                   dm.tex_count() ? (int)(dm.tex_by_id(0) - p0) : -1,
                                   dm.transform_mat(0) ? (int)(dm.transform_mat(0) - p0) : -1,
                                   dm.restricted_transform(0) ? (int)(dm.restricted_transform(0) - p0) : -1,
                                   dm.full_size(), dm.get_mesh_id()};
    out.put_i32(base + ".layout", layout);
    k++;
  }
  out.put_i32("n_dmeshes", {k});
}

// The coordinates the reference's derivative tests draw
// (random_unique_indices, src/tests.cpp:512-541): `cnt` of [from, to) --
// all of them when the range is no larger; else one candidate per stride
// of (to - from) / min(4 cnt, to - from), offset by rand() % stride, then
// std::random_shuffle and the first `cnt`.  It draws from the C library's
// rand() exactly as the test binary does, so called in the tests' order
// from a fresh process it returns the tests' own coordinates.
static std::vector<int> test_coordinates(int from, int to, int cnt) {
  std::vector<int> all;
  if (cnt <= 0) return all;
  if (to - from <= cnt) {
    for (int i = from; i < to; i++) all.push_back(i);
    return all;
  }
  const int stride = (to - from) / std::min(4 * cnt, to - from);
  for (int i = from; i < to; i += stride) all.push_back(stride == 1 ? i : i + std::rand() % stride);
  std::random_shuffle(all.begin(), all.end());
  all.resize(cnt);
  return all;
}

// A mesh with every attribute it has (a prepared scene's mesh after
// restore_meshes), under `prefix`.
static void mesh_out(kv::File& out, const std::string& b, const TriangleMesh& mesh) {
  auto put3 = [&](const char* name, const std::vector<float3>& a) {
    if (a.empty()) return;
    std::vector<float> v;
    for (auto& p : a) { v.push_back(p.x); v.push_back(p.y); v.push_back(p.z); }
    out.put_f32(b + name, v);
  };
  put3("vertices", mesh.vertices);
  put3("colors", mesh.colors);
  put3("normals", mesh.normals);
  put3("tangents", mesh.tangents);
  if (!mesh.tc.empty()) {
    std::vector<float> v;
    for (auto& p : mesh.tc) { v.push_back(p.x); v.push_back(p.y); }
    out.put_f32(b + "tc", v);
  }
  out.put_u32(b + "indices", std::vector<uint32_t>(mesh.indices.begin(), mesh.indices.end()));
  if (!mesh.textures.empty()) {
    const CPUTexture& t = mesh.textures[0];
    out.put_f32(b + "tex", t.m_data);
    out.put_i32(b + "tex_shape", {t.w, t.h, t.channels});
  }
}

static void scene_out(kv::File& out, const std::string& prefix, const Scene& s) {
  for (size_t m = 0; m < s.get_meshes().size(); m++) {
    const TriangleMesh& mesh = s.get_mesh(m);
    std::string b = prefix + "m" + std::to_string(m) + ".";
    std::vector<float> v;
    for (auto& p : mesh.vertices) { v.push_back(p.x); v.push_back(p.y); v.push_back(p.z); }
    out.put_f32(b + "vertices", v);
    std::vector<float> c;
    for (auto& p : mesh.colors) { c.push_back(p.x); c.push_back(p.y); c.push_back(p.z); }
    out.put_f32(b + "colors", c);
    if (!mesh.textures.empty()) out.put_f32(b + "tex", mesh.textures[0].m_data);
    std::vector<float> t;
    for (auto& M : s.get_transform(m)) { auto mv = mat_to_vec(M); t.insert(t.end(), mv.begin(), mv.end()); }
    out.put_f32(b + "transforms", t);
    if (s.get_instancing_type(m) == Scene::RESTRICTED_TRANSFORM) {
      std::vector<float> r;
      for (auto& R : s.get_restricted_transform(m)) {
        const float q[7] = {R.translate.x, R.translate.y, R.translate.z, R.rotate.x, R.rotate.y, R.rotate.z, R.scale};
        r.insert(r.end(), q, q + 7);
      }
      out.put_f32(b + "restricted", r);
    }
  }
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_driver in.kv out.kv\n");
    return 2;
  }
  kv::File in = kv::File::load(argv[1]);
  kv::File out;
  const int task = in.i("task");
  const SHADING_MODEL mode = (SHADING_MODEL)in.i("mode", 2);
  const int spp = in.i("spp", 16);

  if (task == 0) {  // camera matrices
    auto cams = build_cams(in);
    for (size_t i = 0; i < cams.size(); i++) {
      std::string b = "cam" + std::to_string(i) + ".";
      out.put_f32(b + "worldview", mat_to_vec(cams[i].mWorldView));
      out.put_f32(b + "proj", mat_to_vec(cams[i].mProj));
      out.put_f32(b + "wvp", std::vector<float>(cams[i].mWVP, cams[i].mWVP + 16));
      out.put_f32(b + "proj_inv", mat_to_vec(LiteMath::inverse4x4(cams[i].mProj)));
      out.put_f32(b + "wv_inv", mat_to_vec(LiteMath::inverse4x4(cams[i].mWorldView)));
    }
  } else if (task == 1) {  // per-sample nearest hits
    Scene scene;
    build_scene(in, scene);
    auto cams = build_cams(in);
    scene.prepare_for_render();
    auto tracer = MakeRayTracer3D("");
    tracer->Init(&scene);
    tracer->SetCamera(cams[0]);
    auto xy = in.vec<float>("hit_xy");
    size_t n = xy.size() / 2;
    std::vector<uint32_t> prim(n), inst(n), geom(n);
    std::vector<float> t(n), u(n), v(n), rp(3 * n), rd(3 * n);
    for (size_t i = 0; i < n; i++) {
      float3 pos, dir;
      SurfaceInfo s = tracer->CastSingleRay(xy[2 * i], xy[2 * i + 1], &pos, &dir);
      prim[i] = s.primId; inst[i] = s.instId; geom[i] = s.geomId;
      t[i] = s.t; u[i] = s.u; v[i] = s.v;
      rp[3 * i] = pos.x; rp[3 * i + 1] = pos.y; rp[3 * i + 2] = pos.z;
      rd[3 * i] = dir.x; rd[3 * i + 1] = dir.y; rd[3 * i + 2] = dir.z;
    }
    out.put_u32("prim", prim); out.put_u32("inst", inst); out.put_u32("geom", geom);
    out.put_f32("t", t); out.put_f32("u", u); out.put_f32("v", v);
    out.put_f32("ray_pos", rp); out.put_f32("ray_dir", rd);
  } else if (task == 2 || task == 3 || task == 4) {
    Scene scene;
    build_scene(in, scene);
    auto cams = build_cams(in);
    auto dr = make_renderer(in, mode, spp);
    auto t0 = std::chrono::steady_clock::now();
    if (task == 2) {
      std::vector<Img> imgs(cams.size());
      for (size_t i = 0; i < cams.size(); i++) imgs[i].resize((int)cams[i].width, (int)cams[i].height);
      dr->commit(scene);
      // repeats > 1 (a random model such as PATH_TEST): the mean image of
      // that many renders and the unbiased per-value variance across them
      const int repeats = in.i("repeats", 1);
      std::vector<double> sum, sum2;
      for (int r = 0; r < repeats; r++) {
        dr->render(scene, cams.data(), imgs.data(), (int)cams.size());
        if (repeats == 1) break;
        size_t k = 0;
        for (auto& im : imgs) {
          const float* p = (const float*)im.data();
          const size_t n = 3 * (size_t)im.width() * im.height();
          sum.resize(k + n, 0.0);
          sum2.resize(k + n, 0.0);
          for (size_t j = 0; j < n; j++, k++) {
            sum[k] += p[j];
            sum2[k] += (double)p[j] * p[j];
          }
        }
      }
      if (repeats == 1) {
        images_out(out, "images", imgs);
      } else {
        std::vector<float> mean(sum.size()), var(sum.size());
        for (size_t j = 0; j < sum.size(); j++) {
          const double m = sum[j] / repeats;
          mean[j] = (float)m;
          var[j] = (float)std::max(0.0, (sum2[j] - repeats * m * m) / (repeats - 1));
        }
        out.put_f32("images", mean);
        out.put_f32("images_var", var);
      }
    } else {
      std::vector<int> ids;
      for (int32_t x : in.vec<int32_t>("dmesh_ids")) ids.push_back(x);
      DScene ds(scene, layout_mode(mode), ids);
      const int edge_samples = in.i("edge_samples");
      if (task == 3) {
        std::vector<Img> adj;
        images_in(in, "adjoints", cams, adj);
        dr->commit(scene);
        dr->d_render(scene, cams.data(), adj.data(), (int)cams.size(), edge_samples, ds);
      } else {
        std::vector<Img> tgt, imgs(cams.size());
        images_in(in, "targets", cams, tgt);
        float loss = dr->d_render_and_compare(scene, cams.data(), tgt.data(), (int)cams.size(), edge_samples, ds, imgs.data());
        out.put_f32("loss", {loss});
        images_out(out, "images", imgs);
      }
      dscene_out(out, ds);
    }
    auto t1 = std::chrono::steady_clock::now();
    out.put_f64("seconds", {std::chrono::duration<double>(t1 - t0).count()});
  } else if (task == 5) {  // optimisation trajectory
    Scene scene;
    build_scene(in, scene);
    auto cams = build_cams(in);
    std::vector<Img> tgt;
    images_in(in, "targets", cams, tgt);
    auto dr = make_renderer(in, mode, spp);
    OptimizerParameters p((OptimizerParameters::OPT_ALGORITHM)in.i("opt_alg", 4));
    p.position_lr = in.f("opt_pos_lr", p.position_lr);
    p.textures_lr = in.f("opt_tex_lr", p.textures_lr);
    p.transforms_lr = in.f("opt_tfm_lr", p.transforms_lr);
    p.base_lr = in.f("opt_base_lr", p.base_lr);
    p.flags = in.i("opt_flags", p.flags);
    p.decayPeriod = in.i("opt_decay_period", p.decayPeriod);
    p.decay_mult = in.f("opt_decay_mult", p.decay_mult);
    p.verbose = false;
    p.differentiable_mesh_ids.clear();
    for (int32_t x : in.vec<int32_t>("dmesh_ids")) p.differentiable_mesh_ids.push_back(x);
    std::shared_ptr<IOptimizer> opt(CreateSimpleOptimizer());
#ifdef DRGB_WITH_GPU
    if (in.i("backend", 0) == 2) opt = CreateGpuOptimizer();
#endif
    opt->Init(scene, dr, cams.data(), tgt.data(), (int)cams.size(), p);
    std::vector<Scene> dump;
    float err = 0.f;
    auto t0 = std::chrono::steady_clock::now();
    opt->Run((size_t)in.i("iters"), err, &dump);
    auto t1 = std::chrono::steady_clock::now();
    out.put_f32("final_error", {err});
    out.put_f64("seconds", {std::chrono::duration<double>(t1 - t0).count()});
    out.put_i32("n_iters", {(int)dump.size()});
    for (size_t k = 0; k < dump.size(); k++) scene_out(out, "it" + std::to_string(k) + ".", dump[k]);
  } else if (task == 6) {  // prng streams
    auto seeds = in.vec<int32_t>("prng_seeds");
    int cnt = in.i("prng_count");
    std::vector<float> vals;
    for (int s : seeds) {
      prng::RandomGen g = prng::RandomGenInit(s);
      for (int k = 0; k < cnt; k++) vals.push_back(prng::rndFloat(&g));
    }
    out.put_f32("prng", vals);
  } else if (task == 7) {  // Hammersley points
    int n = in.i("ham_n");
    std::vector<float> h(2 * n);
    qmc::planeHammersley(h.data(), n);
    out.put_f32("ham", h);
  } else if (task == 8) {  // a VSGF mesh through the reference's loader (common_src/cmesh.cpp:139-170)
    std::string path;
    for (int32_t ch : in.vec<int32_t>("path")) path.push_back((char)ch);
    mesh_utils::SimpleMesh m = mesh_utils::LoadMeshFromVSGF(path.c_str());
    auto flat = [](const void* p, size_t n) {
      const float* f = static_cast<const float*>(p);
      return std::vector<float>(f, f + n);
    };
    out.put_f32("pos4", flat(m.vPos4f.data(), 4 * m.vPos4f.size()));
    out.put_f32("norm4", flat(m.vNorm4f.data(), 4 * m.vNorm4f.size()));
    out.put_f32("tc2", flat(m.vTexCoord2f.data(), 2 * m.vTexCoord2f.size()));
    out.put_u32("indices", std::vector<uint32_t>(m.indices.begin(), m.indices.end()));
  } else if (task == 9) {
    // The scenes and camera of the reference's derivative tests 1.1-1.5
    // (src/tests.cpp:31-107): initial and target meshes as the tests build
    // them from src/scenes.cpp, after their transforms and restore_meshes.
    CamInfo camera;
    camera.width = 256.0f;
    camera.height = 256.0f;
    camera.mWorldView = LiteMath::translate4x4(float3(0, 0, -3));
    camera.mProj = LiteMath::perspectiveMatrix(45.0f, camera.width / camera.height, 0.1f, 100.0f);
    camera.commit();
    out.put_f32("cam.worldview", mat_to_vec(camera.mWorldView));
    out.put_f32("cam.proj", mat_to_vec(camera.mProj));
    for (int k = 1; k <= 5; k++) {
      TriangleMesh initialMesh, targetMesh;
      Scene initialScene, targetScene;
      if (k == 1) scn03_Triangle3D_White(initialMesh, targetMesh);
      if (k == 2 || k == 4) scn05_Pyramid3D(initialMesh, targetMesh);
      if (k == 3 || k == 5) scn09_Sphere3D_Textured(initialMesh, targetMesh);
      if (k == 3) transform(initialMesh, LiteMath::translate4x4(float3(0, +0.2f, 0.0f)));
      initialScene.add_mesh(initialMesh);
      targetScene.add_mesh(targetMesh);
      if (k == 3) {
        initialScene.restore_meshes(false, false, true);
        targetScene.restore_meshes(false, false, true);
      }
      const std::string b = "t1" + std::to_string(k) + ".";
      mesh_out(out, b + "initial.", initialScene.get_mesh(0));
      mesh_out(out, b + "target.", targetScene.get_mesh(0));
      // the vertices (at most 100) and texels (1.5: 250) the test checks,
      // drawn in the order test_base_derivatives draws them
      const TriangleMesh& m = initialScene.get_mesh(0);
      const int max_v = k == 5 ? 0 : 100, max_t = k == 5 ? 250 : 0;
      auto verts = test_coordinates(0, m.vertex_count(), max_v);
      out.put_i32(b + "test_vertices", std::vector<int32_t>(verts.begin(), verts.end()));
      if (max_t > 0 && !m.textures.empty()) {
        auto texels = test_coordinates(0, m.textures[0].w * m.textures[0].h, max_t);
        out.put_i32(b + "test_texels", std::vector<int32_t>(texels.begin(), texels.end()));
      }
    }
  } else {
    std::fprintf(stderr, "unknown task %d\n", task);
    return 2;
  }
  out.save(argv[2]);
  return 0;
}
