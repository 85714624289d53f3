// Host-side set-up of a render job: scene upload and flattening tables,
// cameras, gradient layout, the edge list and the replayed random streams.
// Host arithmetic that must match the reference (camera matrices,
// Hammersley points, the edge-sampler streams) is compiled without
// floating-point contraction (-Xcompiler -ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>

#include "engine.h"

namespace drgb {

// ---------------------------------------------------------------------------
// Camera: CamInfo (common_src/camera.h:9-44) with lookAt / perspectiveMatrix
// (LiteMath.h:1679-1729); BruteForce3D::SetCamera inverses
// (raytrace_src/raytrace3d_bf.cpp:93-100).
// ---------------------------------------------------------------------------
namespace {
struct H3 {
  float x, y, z;
};
H3 h3(float x, float y, float z) { return H3{x, y, z}; }
float hdot(H3 a, H3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
H3 hnorm(H3 a) {
  const float inv = 1.0f / std::sqrt(hdot(a, a));
  return h3(a.x * inv, a.y * inv, a.z * inv);
}
H3 hcross(H3 a, H3 b) {
  const float dx = a.x * b.y - a.y * b.x, dy = a.y * b.z - a.z * b.y, dz = a.z * b.x - a.x * b.z;
  return h3(dy, dz, dx);
}
void mat_vec4(const float* B, const float* V, float* R) {
  for (int i = 0; i < 4; i++) R[i] = V[0] * B[i] + V[1] * B[4 + i] + V[2] * B[8 + i] + V[3] * B[12 + i];
}
void mat_mul(const float* a, const float* b, float* out) {
  float tmp[16];
  for (int c = 0; c < 4; c++) mat_vec4(a, b + 4 * c, tmp + 4 * c);
  std::memcpy(out, tmp, sizeof(tmp));
}
}  // namespace

void camera_look_at(const float* o, const float* t, const float* u, float width, float height, float fov_rad,
                    float znear, float zfar, drgb_camera* out) {
  const float DEG_TO_RAD = 3.14159265358979323846f / 180.0f;
  const float fovy = fov_rad / DEG_TO_RAD;
  const float aspect = width / height;
  // tan through double: correctly rounded for these arguments on every host
  const float ymax = znear * (float)std::tan((double)(fovy * 3.14159265358979323846f / 360.0f));
  const float xmax = ymax * aspect;
  const float left = -xmax, right = +xmax, bottom = -ymax, top = +ymax;
  const float temp = 2.0f * znear, temp2 = right - left, temp3 = top - bottom, temp4 = zfar - znear;
  const float P[16] = {temp / temp2, 0.0f, 0.0f, 0.0f, 0.0f, temp / temp3, 0.0f, 0.0f,
                       (right + left) / temp2, (top + bottom) / temp3, (-zfar - znear) / temp4, -1.0f,
                       0.0f, 0.0f, (-temp * zfar) / temp4, 0.0f};
  const H3 eye = h3(o[0], o[1], o[2]);
  H3 z = hnorm(h3(o[0] - t[0], o[1] - t[1], o[2] - t[2]));
  H3 y = h3(u[0], u[1], u[2]);
  H3 x = hcross(y, z);
  y = hcross(z, x);
  x = hnorm(x);
  y = hnorm(y);
  const float V[16] = {x.x, y.x, z.x, 0.0f, x.y, y.y, z.y, 0.0f, x.z, y.z, z.z, 0.0f,
                       -x.x * eye.x - x.y * eye.y - x.z * eye.z, -y.x * eye.x - y.y * eye.y - y.z * eye.z,
                       -z.x * eye.x - z.y * eye.y - z.z * eye.z, 1.0f};
  std::memcpy(out->world_view, V, sizeof(V));
  std::memcpy(out->proj, P, sizeof(P));
  out->width = width;
  out->height = height;
}

CamDev make_cam(const drgb_camera& c) {
  CamDev d;
  std::memcpy(d.wv, c.world_view, sizeof(d.wv));
  std::memcpy(d.proj, c.proj, sizeof(d.proj));
  mat_mul(c.proj, c.world_view, d.wvp);  // CamInfo::commit: mProj*mWorldView
  mat_inverse44(c.proj, d.proj_inv);
  mat_inverse44(c.world_view, d.wv_inv);
  d.width = c.width;
  d.height = c.height;
  // camera_ray's origin: mat_pt(wv_inv, (0,0,0)) in the device's operation
  // order (host code is built without contraction, so the bits agree)
  const float z = 0.0f, one = 1.0f;
  for (int i = 0; i < 3; i++)
    d.ro[i] = z * d.wv_inv[i] + z * d.wv_inv[4 + i] + z * d.wv_inv[8 + i] + one * d.wv_inv[12 + i];
  auto pow2_inv = [](float w) {
    int e = 0;
    return (w > 0.0f && std::frexp(w, &e) == 0.5f) ? 1.0f / w : 0.0f;
  };
  d.inv_w = pow2_inv(c.width);
  d.inv_h = pow2_inv(c.height);
  return d;
}

// TransformR::to_mat (common_src/scene.h:99-104): translate4x4(t) *
// rotate4x4Z(rz) * rotate4x4Y(ry) * rotate4x4X(rx) * scale4x4(s), the
// products left to right in LiteMath's order (LiteMath.h:1474-1549).
void restricted_to_mat(const float* p, float* out) {
  auto ident = [](float* m) {
    std::fill(m, m + 16, 0.0f);
    m[0] = m[5] = m[10] = m[15] = 1.0f;
  };
  float T[16], Rz[16], Ry[16], Rx[16], S[16], a[16], b[16];
  ident(T);
  T[12] = p[0]; T[13] = p[1]; T[14] = p[2];
  ident(Rz);
  Rz[0] = std::cos(p[5]); Rz[1] = std::sin(p[5]); Rz[4] = -std::sin(p[5]); Rz[5] = std::cos(p[5]);
  ident(Ry);
  Ry[0] = std::cos(p[4]); Ry[2] = -std::sin(p[4]); Ry[8] = std::sin(p[4]); Ry[10] = std::cos(p[4]);
  ident(Rx);
  Rx[5] = std::cos(p[3]); Rx[6] = std::sin(p[3]); Rx[9] = -std::sin(p[3]); Rx[10] = std::cos(p[3]);
  ident(S);
  S[0] = S[5] = S[10] = p[6];
  mat_mul(T, Rz, a);
  mat_mul(a, Ry, b);
  mat_mul(b, Rx, a);
  mat_mul(a, S, out);
}

// qmc::planeHammersley (common_src/qmc.cpp:227-243)
static void hammersley(int n, float* out) {
  for (int k = 0; k < n; k++) {
    float u = 0;
    int kk = k;
    for (float p = 0.5f; kk; p *= 0.5f, kk >>= 1)
      if (kk & 1) u += p;
    out[2 * k] = u;
    out[2 * k + 1] = (k + 0.5f) / n;
  }
}

// ---------------------------------------------------------------------------
// Scene upload.
// ---------------------------------------------------------------------------
void upload_scene(Job& J, const drgb_scene_desc* scene, cudaStream_t s) {
  if (!scene || scene->n_meshes < 0 || (scene->n_meshes > 0 && !scene->meshes))
    throw CudaError("scene descriptor is null or malformed", DRGB_ERR_INVALID);
  const int nm = scene->n_meshes;
  // every mesh is checked before anything of the committed scene changes
  for (int m = 0; m < nm; m++) {
    const drgb_mesh_desc& d = scene->meshes[m];
    if (d.n_vertices < 0 || d.n_indices < 0 || d.n_indices % 3 != 0 || (d.n_vertices > 0 && !d.vertices) ||
        (d.n_indices > 0 && !d.indices))
      throw CudaError("mesh " + std::to_string(m) + ": bad vertex/index arrays", DRGB_ERR_INVALID);
    if (d.n_instances > 1 && !d.transforms && !d.restricted)
      throw CudaError("mesh " + std::to_string(m) + ": several instances need transforms", DRGB_ERR_INVALID);
    const bool tex = d.texture && d.tex_w > 0 && d.tex_h > 0;
    if (tex && d.tex_channels != 3) throw CudaError("textures must have 3 channels", DRGB_ERR_INVALID);
    if (model_has_tex(J.mode) && !tex)
      throw CudaError("mesh " + std::to_string(m) + ": the shading model needs a texture", DRGB_ERR_INVALID);
    if (model_has_tex(J.mode) && !d.tc)
      throw CudaError("mesh " + std::to_string(m) + ": the shading model needs texture coordinates", DRGB_ERR_INVALID);
  }
  // The same meshes with the same vertex and instance counts and the same
  // index arrays as the committed scene (an optimiser moving vertices): the
  // index check and the triangle tables (blocks, vertex blocks, triangle
  // list) carry over.
  bool same_structure = J.committed && (int)J.meshes.size() == nm;
  for (int m = 0; m < nm && same_structure; m++) {
    const drgb_mesh_desc& d = scene->meshes[m];
    const MeshState& M = J.meshes[m];
    same_structure = M.nv == d.n_vertices && M.ni == d.n_indices &&
                     M.n_inst == (d.n_instances <= 0 ? 1 : d.n_instances) &&
                     (int)M.h_indices.size() == d.n_indices &&
                     (d.n_indices == 0 ||
                      std::memcmp(M.h_indices.data(), d.indices, sizeof(uint32_t) * (size_t)d.n_indices) == 0);
  }
  if (!same_structure)
    for (int m = 0; m < nm; m++) {
      const drgb_mesh_desc& d = scene->meshes[m];
      for (int i = 0; i < d.n_indices; i++)
        if (d.indices[i] >= (uint32_t)d.n_vertices)
          throw CudaError("mesh " + std::to_string(m) + ": index out of range", DRGB_ERR_INVALID);
    }
  rebuild_bvh_discard(J);  // a host build in progress reads the triangle lists replaced here
  // from here on the committed scene changes: a failure part-way (a device
  // error) leaves no scene committed, and the next commit rebuilds everything
  J.committed = false;
  // The meshes' device buffers are kept from the last commit and reused where
  // the sizes agree: a commit of the same meshes (the reference commits the
  // scene on every d_render_and_compare, drender.h:176) frees and allocates
  // nothing (cudaFree waits for the whole device).  Uploads are ordered on
  // the renderer's stream behind any work that still reads them.
  J.meshes.resize(nm);
  if (!same_structure) J.h_blocks.clear();
  std::vector<int> vblock;
  std::vector<int4> tri_v;
  int voff = 0, toff = 0;
  for (int m = 0; m < nm; m++) {
    const drgb_mesh_desc& d = scene->meshes[m];
    MeshState& M = J.meshes[m];
    const int ninst = d.n_instances <= 0 ? 1 : d.n_instances;
    M.nv = d.n_vertices;
    M.ni = d.n_indices;
    M.n_inst = ninst;
    M.vertices.upload(d.vertices, 3 * (size_t)d.n_vertices, s);
    M.has_colors = d.colors != nullptr;
    M.has_tc = d.tc != nullptr;
    M.has_normals = d.normals != nullptr;
    M.has_tangents = d.tangents != nullptr;
    if (M.has_colors) M.colors.upload(d.colors, 3 * (size_t)d.n_vertices, s);
    else M.colors.reset();
    if (M.has_tc) M.tc.upload(d.tc, 2 * (size_t)d.n_vertices, s);
    else M.tc.reset();
    if (M.has_normals) M.normals.upload(d.normals, 3 * (size_t)d.n_vertices, s);
    else M.normals.reset();
    if (M.has_tangents) M.tangents.upload(d.tangents, 3 * (size_t)d.n_vertices, s);
    else M.tangents.reset();
    if (!same_structure) M.h_indices.assign(d.indices, d.indices + d.n_indices);  // on the device as tri_v
    std::vector<float> tr(16 * (size_t)ninst, 0.0f);
    M.restricted = d.restricted != nullptr;
    if (M.restricted) {
      for (int j = 0; j < ninst; j++) restricted_to_mat(d.restricted + 7 * j, &tr[16 * j]);
      M.rparams.upload(d.restricted, 7 * (size_t)ninst, s);
    } else if (d.transforms) {
      std::memcpy(tr.data(), d.transforms, sizeof(float) * 16 * ninst);
    } else {
      for (int j = 0; j < ninst; j++) tr[16 * j + 0] = tr[16 * j + 5] = tr[16 * j + 10] = tr[16 * j + 15] = 1.0f;
    }
    if (!M.restricted) M.rparams.reset();
    M.h_transforms = tr;
    M.transforms.upload(tr.data(), tr.size(), s);
    if (d.texture && d.tex_w > 0 && d.tex_h > 0) {
      M.tex_w = d.tex_w;
      M.tex_h = d.tex_h;
      M.tex_c = d.tex_channels;
      M.texture.upload(d.texture, (size_t)d.tex_w * d.tex_h * d.tex_channels, s);
    } else {
      M.tex_w = M.tex_h = M.tex_c = 0;
      M.texture.reset();
    }
    for (int j = 0; j < ninst && !same_structure; j++) {
      const int b = (int)J.h_blocks.size();
      J.h_blocks.push_back(BlockDev{voff, toff, m, j});
      for (int k = 0; k < d.n_vertices; k++) vblock.push_back(b);
      for (int p = 0; p < d.n_indices / 3; p++)
        tri_v.push_back(make_int4(voff + (int)d.indices[3 * p], voff + (int)d.indices[3 * p + 1],
                                  voff + (int)d.indices[3 * p + 2], b));
      voff += d.n_vertices;
      toff += d.n_indices / 3;
    }
  }
  bool same_topology = true;
  if (!same_structure) {
    J.n_vertices = voff;
    J.n_tris = toff;
    J.n_blocks = (int)J.h_blocks.size();
    upload_changed(J.blocks, J.up_blocks, J.h_blocks.data(), J.h_blocks.size(), s);
    upload_changed(J.vblock, J.up_vblock, vblock.data(), vblock.size(), s);
    // the same triangles (global vertex ids and blocks) keep the edge list
    same_topology = tri_v.size() == J.h_tri_v.size() &&
                    (tri_v.empty() || std::memcmp(tri_v.data(), J.h_tri_v.data(), sizeof(int4) * tri_v.size()) == 0);
    if (!same_topology || !J.tri_v.p || J.tri_v.n != tri_v.size()) J.tri_v.upload(tri_v.data(), tri_v.size(), s);
    J.h_tri_v.swap(tri_v);  // kept for the hierarchy builders and their topology cache
  }
  std::vector<MeshSrc> src(nm);
  std::vector<const float*> trs(nm);
  for (int m = 0; m < nm; m++) {
    const MeshState& M = J.meshes[m];
    src[m] = MeshSrc{M.vertices.p, M.has_colors ? M.colors.p : nullptr, M.has_normals ? M.normals.p : nullptr,
                     M.has_tc ? M.tc.p : nullptr, M.has_tangents ? M.tangents.p : nullptr};
    trs[m] = M.transforms.p;
  }
  upload_changed(J.src_tab, J.up_src_tab, src.data(), src.size(), s);
  upload_changed(J.tr_tab, J.up_tr_tab, trs.data(), trs.size(), s);
  const size_t nv = std::max(1, J.n_vertices);
  J.pos.alloc(nv);
  J.orig.alloc(nv);
  J.col.alloc(nv);
  J.nrm.alloc(nv);
  if (J.mode == PATH_TEST) J.tan.alloc(nv);  // the path model's shading frames
  J.tc.alloc(nv);
  J.block_tr.alloc(32 * (size_t)std::max(1, J.n_blocks));
  // inverse transforms of mesh 0 (Scene::get_transform_inv(0), kept from the
  // first commit: prepare_for_render appends, scene_utils.cpp:118-129)
  if (nm > 0) {
    // The edge term indexes this table by the instance of any mesh; instances
    // beyond mesh 0's (an out-of-range read in the reference) get the
    // identity, so that every index stays inside the table.
    int max_inst = 1;
    for (int m = 0; m < nm; m++) max_inst = std::max(max_inst, J.meshes[m].n_inst);
    std::vector<float> tr(16 * (size_t)max_inst, 0.0f), inv(tr.size(), 0.0f);
    const MeshState& M0 = J.meshes[0];
    for (int j = 0; j < max_inst; j++) {
      if (j < M0.n_inst) std::memcpy(&tr[16 * j], &M0.h_transforms[16 * j], 16 * sizeof(float));
      else tr[16 * j] = tr[16 * j + 5] = tr[16 * j + 10] = tr[16 * j + 15] = 1.0f;
      mat_inverse44(&tr[16 * j], &inv[16 * j]);
    }
    upload_changed(J.tr_inv0, J.up_tr_inv0, inv.data(), inv.size(), s);
  }
  if (!same_topology) {
    J.edge_ids_key.clear();
    J.n_edges = 0;
  }
  J.committed = true;
}

void setup_views(Job& J, const drgb_camera* cams, int n_views) {
  if (n_views <= 0 || !cams) throw CudaError("need at least one camera", DRGB_ERR_INVALID);
  J.h_cams.resize(n_views);
  for (int i = 0; i < n_views; i++) {
    if (!(cams[i].width >= 1.0f) || !(cams[i].height >= 1.0f))
      throw CudaError("camera size must be positive", DRGB_ERR_INVALID);
    J.h_cams[i] = make_cam(cams[i]);
  }
  J.n_views = n_views;
  J.W = (int)cams[0].width;
  J.H = (int)cams[0].height;
}

int64_t compute_layout(const Job& J, const int32_t* ids, int n_ids, std::vector<DLayout>& out,
                       int64_t* alloc_total) {
  if (n_ids < 0 || n_ids > 16 || (n_ids > 0 && !ids)) throw CudaError("bad differentiable mesh ids", DRGB_ERR_INVALID);
  out.clear();
  int64_t off = 0;
  for (int k = 0; k < n_ids; k++) {
    const int id = ids[k];
    if (id < 0 || id >= (int)J.meshes.size()) throw CudaError("differentiable mesh id out of range", DRGB_ERR_INVALID);
    for (int q = 0; q < k; q++)
      if (ids[q] == id) throw CudaError("duplicate differentiable mesh id", DRGB_ERR_INVALID);
    const MeshState& M = J.meshes[id];
    DLayout L;
    L.mesh_id = id;
    L.vertices = M.nv;
    L.instances = M.n_inst;
    int o = 0;
    L.pos_off = o;
    o += 3 * M.nv;
    if (model_has_color(J.mode)) { L.color_off = o; o += 3 * M.nv; }
    if (model_has_tex(J.mode) && M.texture.p) { L.tex_off = o; o += M.tex_w * M.tex_h * M.tex_c; }
    if (M.restricted) {
      L.rt_off = o;
      o += 7 * M.n_inst;
    } else {
      L.tr_off = o;
      o += 12 * M.n_inst;
    }
    L.full = o;
    L.base = off;
    off += o;
    out.push_back(L);
  }
  // scratch matrix blocks of the restricted meshes, after the public vector
  int64_t scratch = off;
  for (DLayout& L : out)
    if (L.rt_off >= 0) {
      L.tr_off = (int)(scratch - L.base);
      scratch += 12 * (int64_t)L.instances;
    }
  if (alloc_total) *alloc_total = scratch;
  return off;
}

// Unique edges of the meshes of `lay` ordered by (v0, v1) global ids, the
// first inserted kept on duplicates (std::set<Edge>, drender.h:244-299);
// insertion runs over meshes, then instances, then triangles.  `tris` (may
// be null) receives the flattened ids of the first two triangles that share
// each edge (-1 where an edge has only one: a boundary edge).
void edge_list(const Job& J, const std::vector<DLayout>& lay, std::vector<int4>& ed, std::vector<int2>& mi,
               std::vector<int2>* tris) {
  std::vector<int> key;
  for (auto& L : lay) key.push_back(L.mesh_id);
  std::sort(key.begin(), key.end());
  struct E {
    int v0, v1, vn0, vn1, mesh, inst, tri;
  };
  std::vector<E> all;
  for (int m = 0; m < (int)J.meshes.size(); m++) {
    if (!std::binary_search(key.begin(), key.end(), m)) continue;
    const MeshState& M = J.meshes[m];
    for (int j = 0; j < M.n_inst; j++) {
      int b = -1;
      for (int q = 0; q < J.n_blocks; q++)
        if (J.h_blocks[q].mesh == m && J.h_blocks[q].inst == j) b = q;
      const int off = J.h_blocks[b].vert_off, toff = J.h_blocks[b].tri_off;
      for (int k = 0; k + 2 < M.ni; k += 3) {
        const int n[3] = {(int)M.h_indices[k], (int)M.h_indices[k + 1], (int)M.h_indices[k + 2]};
        for (int e = 0; e < 3; e++) {
          const int a = n[e], c = n[(e + 1) % 3];
          const int ga = off + a, gc = off + c;
          if (ga < gc) all.push_back(E{ga, gc, a, c, m, j, toff + k / 3});
          else all.push_back(E{gc, ga, c, a, m, j, toff + k / 3});
        }
      }
    }
  }
  std::stable_sort(all.begin(), all.end(), [](const E& x, const E& y) {
    return x.v0 != y.v0 ? x.v0 < y.v0 : x.v1 < y.v1;
  });
  ed.clear();
  mi.clear();
  if (tris) tris->clear();
  for (const E& e : all) {
    if (!ed.empty() && ed.back().x == e.v0 && ed.back().y == e.v1) {
      if (tris && tris->back().y < 0) tris->back().y = e.tri;
      continue;
    }
    ed.push_back(make_int4(e.v0, e.v1, e.vn0, e.vn1));
    mi.push_back(make_int2(e.mesh, e.inst));
    if (tris) tris->push_back(make_int2(e.tri, -1));
  }
}

void build_edges(Job& J) {
  std::vector<int> key;
  for (auto& L : J.dlay) key.push_back(L.mesh_id);
  std::sort(key.begin(), key.end());
  if (key == J.edge_ids_key && (J.n_edges > 0 || key.empty())) return;
  std::vector<int4> ed;
  std::vector<int2> mi, tris;
  edge_list(J, J.dlay, ed, mi, &tris);
  J.n_edges = (int)ed.size();
  J.edges.upload(ed.data(), ed.size(), 0);
  J.edge_mi.upload(mi.data(), mi.size(), 0);
  J.edge_tris.upload(tris.data(), tris.size(), 0);
  DRGB_CUDA(cudaStreamSynchronize(0));
  J.edge_ids_key = key;
}

int first_block(const Job& J, int mesh) {
  for (int b = 0; b < J.n_blocks; b++)
    if (J.h_blocks[b].mesh == mesh) return b;
  return 0;
}

void set_dscene(Job& J, const int32_t* ids, int n_ids, cudaStream_t s) {
  J.grad_total = compute_layout(J, ids, n_ids, J.dlay, &J.grad_alloc);
  J.dmesh_ids.assign(ids, ids + n_ids);
  J.grad.reserve(std::max<int64_t>(1, J.grad_alloc));
  std::vector<MeshDev> md(J.meshes.size(), MeshDev{});
  for (size_t m = 0; m < J.meshes.size(); m++) {
    const MeshState& M = J.meshes[m];
    MeshDev& d = md[m];
    d.tex = M.texture.p;
    d.tex_w = M.tex_w;
    d.tex_h = M.tex_h;
    d.tex_c = M.tex_c;
    d.dslot = -1;
    d.g_base = 0;
    d.pos_off = 0;
    d.color_off = d.tex_off = -1;
    d.tr_off = 0;
    d.n_vertices = M.nv;
    d.n_instances = M.n_inst;
    d.block0 = first_block(J, (int)m);
  }
  for (size_t k = 0; k < J.dlay.size(); k++) {
    const DLayout& L = J.dlay[k];
    MeshDev& d = md[L.mesh_id];
    d.dslot = (int)k;
    d.g_base = L.base;
    d.pos_off = L.pos_off;
    d.color_off = L.color_off;
    d.tex_off = L.tex_off;
    d.tr_off = L.tr_off;
  }
  // the table changes when the meshes or the differentiated set do: repeated
  // calls on one scene upload nothing; an upload is ordered on the stream
  // behind the work that still reads the previous table
  if (J.meshdev.p && J.meshdev.n == md.size() && J.h_meshdev.size() == md.size() &&
      std::memcmp(J.h_meshdev.data(), md.data(), sizeof(MeshDev) * md.size()) == 0)
    return;
  J.meshdev.upload(md.data(), md.size(), s);
  J.h_meshdev = md;
}

// Pixel tile of one warp: at most 32 samples (one pixel when a pixel has
// more); maximise pixels, prefer square.
void choose_tile(int S, int& tw, int& th) {
  const int P = std::max(1, 32 / std::max(1, S));
  int best = 0;
  tw = th = 1;
  for (int h = 1; h <= P; h++) {
    const int w = P / h;
    if (w < h) break;
    const int area = w * h;
    if (area > best || (area == best && (w - h) < (tw - th))) {
      best = area;
      tw = w;
      th = h;
    }
  }
}

void sync_dev(Job& J) {
  JobDev& d = J.dev;
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
  d.meshes = J.meshdev.p;
  d.tr_inv0 = J.tr_inv0.p;
  d.block_tr = J.block_tr.p;
  d.nodes = J.nodes.p;
  d.nodes4 = J.nodes4.p;
  d.tri = J.tri.p;
  d.leaf_of = J.leaf_of.p;
  // the binned-SAH topology numbers its top levels first (breadth first)
#ifdef DRGB_TOP_SMEM
  d.top_n = J.topo_builder >= 1 ? std::min(std::max(J.n_tris - 1, 0), kTopNodes) : 0;
#else
  d.top_n = 0;
#endif
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
  d.n_views = J.n_views;
  d.cams = J.cams.p;
  d.W = J.W;
  d.H = J.H;
  d.grad = J.grad.p;
  d.err = J.err.p;
  d.images = J.images.p;
  d.img_off = J.img_off.p;
  d.targets = J.targets.p;
  d.adj = J.adj.p;
  d.adj_in = J.adj_in.p;
  d.loss_part = J.loss_part.p;
  d.loss_blk = J.loss_blk.p;
  d.loss_ticket = J.loss_ticket.p;
  d.loss_out = J.loss_out.p;
  d.tile_w = J.tile_w;
  d.tile_h = J.tile_h;
  d.edges = J.edges.p;
  d.edge_mi = J.edge_mi.p;
  d.edge_tris = J.edge_tris.p;
  d.edge_sil = J.edge_sil;
  d.vis_fwd = J.raster_on ? J.vis[0].p : nullptr;
  d.vis_adj = J.raster_on ? J.vis[1].p : nullptr;
  d.vis_uv_fwd = J.raster_on && vis_points(J.mode) ? J.vis_uv[0].p : nullptr;
  d.vis_uv_adj = J.raster_on && vis_points(J.mode) ? J.vis_uv[1].p : nullptr;
  d.ra_state = J.ra_state.p;
  d.ra_tiles = J.raster_on ? J.ra_tiles.p : nullptr;
  d.ra_list = J.ra_list.p;
  d.ra_rec = J.ra_rec.p;
  raster_tile(J.S, d.ra_tw, d.ra_th);
  {
    int W = 1, H = 1;
    for (auto& c : J.h_cams) {
      W = std::max(W, (int)c.width);
      H = std::max(H, (int)c.height);
    }
    d.ra_ntx = (W + d.ra_tw - 1) / d.ra_tw;
    d.ra_nty = (H + d.ra_th - 1) / d.ra_th;
  }
  d.sh_grid = J.shadow_on ? J.sh_grid.p : nullptr;
  d.sh_cells = J.sh_cells.p;
  d.sh_list = J.sh_list.p;
  d.sh_rec = J.sh_rec.p;
  d.n_edges = J.n_edges;
  d.proj = J.proj.p;
  d.pmf = J.pmf.p;
  d.cdf = J.cdf.p;
  d.queue = J.queue.p;
  d.queue_count = J.queue_count.p;
  d.queue_cap = (int)J.queue.n;
  d.work = nullptr;
  d.det = (J.det && J.rec_key.p) ? 1 : 0;
  d.rec_item_cap = item_record_cap(J.mode, J.tile_w * J.tile_h * J.S);
  d.rec_key = J.rec_key.p;
  d.rec_val = J.rec_val.p;
  d.rec_count = J.rec_count.p;
  d.det_tr = d.det && J.det_tr_key >= 0 ? J.det_tr.p : nullptr;
  d.det_tr_key = J.det_tr_key;
  d.hit_buf = J.hit_buf.p;
}

// ---------------------------------------------------------------------------
// Replayed edge-sampler streams: sample i of OpenMP thread k's static block
// draws (rnd0, rnd1) from prng stream 7777 + k^2 + 1 (drender.h:306-331,
// common_src/qmc.cpp:250-268; libgomp static schedule, 14 threads).  The
// streams restart for every view and every call, so one table serves all.
// ---------------------------------------------------------------------------
static void prng_stream(int seed, int count, float* out) {
  const uint32_t us = (uint32_t)seed;
  uint32_t sx = us * (us * us * 15731u + 74323u) + 871483u;
  uint32_t sy = us * (us * us * 13734u + 37828u) + 234234u;
  for (int i = 0; i < (seed % 7); i++) {
    const uint32_t x = sx * 17u + sy * 13123u;
    sx = (x << 13) ^ x;
    sy ^= (x << 7);
  }
  for (int k = 0; k < count; k++) {
    const uint32_t x = sx * 17u + sy * 13123u;
    sx = (x << 13) ^ x;
    sy ^= (x << 7);
    const uint32_t tmp = (x * (x * x * 15731u + 74323u) + 871483u);
    out[k] = (float)tmp * (1.0f / 4294967296.0f);
  }
}

void edge_random_host(int n, std::vector<float>& h) {
  h.assign(2 * (size_t)std::max(n, 1), 0.0f);
  const int T = 14;
  const int64_t q = n / T, r = n % T;
  for (int k = 0; k < T; k++) {
    const int64_t b = q * k + std::min<int64_t>(k, r);
    const int64_t cnt = q + (k < r ? 1 : 0);
    if (cnt > 0) prng_stream(7777 + k * k + 1, (int)(2 * cnt), h.data() + 2 * b);
  }
}

const float* edge_random_table(int n, cudaStream_t s) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, DevBuf<float>*> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({dev, n});
  if (it != cache.end()) return it->second->p;
  std::vector<float> h;
  edge_random_host(n, h);
  auto* buf = new DevBuf<float>();
  buf->upload(h.data(), h.size(), s);
  DRGB_CUDA(cudaStreamSynchronize(s));
  cache[{dev, n}] = buf;  // lives until process exit; shared by every renderer
  return buf->p;
}

const int* edge_random_order(int n, cudaStream_t s) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, DevBuf<int>*> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({dev, n});
  if (it != cache.end()) return it->second->p;
  std::vector<float> h;
  edge_random_host(n, h);
  std::vector<int> order(std::max(n, 1));
  for (int i = 0; i < (int)order.size(); i++) order[i] = i;
  if (n > 0)
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return h[2 * (size_t)a] < h[2 * (size_t)b]; });
  auto* buf = new DevBuf<int>();
  buf->upload(order.data(), order.size(), s);
  DRGB_CUDA(cudaStreamSynchronize(s));
  cache[{dev, n}] = buf;  // lives until process exit; shared by every renderer
  return buf->p;
}

void init_job_model(Job& J, int mode, int spp) {
  J.mode = mode;
  J.spp = spp;
  J.sq = (int)std::sqrt((float)spp);
  J.S = J.sq * J.sq;
  std::vector<float> h(2 * (size_t)spp);
  hammersley(spp, h.data());
  J.ham.upload(h.data(), h.size(), 0);
  DRGB_CUDA(cudaStreamSynchronize(0));
  choose_tile(J.S, J.tile_w, J.tile_h);
  J.mp.light_pos[0] = J.mp.light_pos[1] = J.mp.light_pos[2] = 3.0f;
  J.mp.light_intensity = 10.0f;
  J.mp.ambient = 0.1f;
  J.mp.path_depth = 2;
  J.mp.seed = 1u;
  J.err.alloc(1);
  DRGB_CUDA(cudaMemset(J.err.p, 0, sizeof(uint32_t)));
  J.loss_out.alloc(1);
  J.queue_count.alloc(2);  // [0] queue entries, [1] shading counter
}

}  // namespace drgb
