// Device-side data layout and math shared by the renderer kernels.
//
// Every translation unit that includes this header is compiled with
// -fmad=false: the reference's CPU arithmetic (x86-64, no FMA contraction) is
// reproduced operation by operation, so that camera rays, hit distances,
// barycentrics and shaded colours are bit-identical to the reference's
// brute-force caster.  Where rounding does not have to match (BVH slab
// tests), fused multiply-adds are requested explicitly with __fmaf_rn.
#pragma once
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

namespace drgb {

// ---------------------------------------------------------------------------
// Shading models: numbering of SHADING_MODEL (src/dmesh.h:16-23) plus two
// models without a reference counterpart.
// ---------------------------------------------------------------------------
enum Model : int {
  SILHOUETTE = 1,
  VERTEX_COLOR = 2,
  TEXTURE_COLOR = 3,
  LAMBERT = 4,
  PHONG = 5,
  GGX = 6,
  PATH_TEST = 7,
  LAMBERT_POINT_VCOLOR = 16,
  PATH_DIFFUSE = 17,
};

__host__ __device__ inline bool model_has_color(int m) {
  return m == VERTEX_COLOR || m == LAMBERT_POINT_VCOLOR || m == PATH_DIFFUSE;
}
__host__ __device__ inline bool model_has_tex(int m) {
  return m == TEXTURE_COLOR || m == LAMBERT || m == PHONG || m == GGX || m == PATH_TEST;
}
// Whether a model's shader reads the camera ray (0: the generic shader, any
// model); vertex colour, texture and silhouette interpolate by u, v alone.
__host__ __device__ constexpr bool model_reads_ray(int m) {
  return !(m == SILHOUETTE || m == VERTEX_COLOR || m == TEXTURE_COLOR);
}
// Models whose samples trace several bounces (random walks of varying length).
__host__ __device__ constexpr bool model_is_path(int m) { return m == PATH_DIFFUSE || m == PATH_TEST; }

constexpr int kStackSize = 96;
constexpr int kEmpty4 = (int)0x80000000;  // unused slot of a 4-wide node
constexpr uint32_t kNoHit = 0xFFFFFFFFu;

// Error flags raised by kernels (never trap): the host reads them after a call.
enum ErrFlag : uint32_t {
  ERR_STACK_OVERFLOW = 1u,
  ERR_TRAVERSAL_LIMIT = 2u,
  ERR_VISIBILITY = 8u,  // a rasterised hit names a triangle the scene does not have
  ERR_BAD_INDEX = 4u,
};

// Camera block: the 82 floats of the oracle's layout (world_view, proj, wvp,
// proj_inv, wv_inv, width, height), computed on the host like CamInfo.
struct CamDev {
  float wv[16];
  float proj[16];
  float wvp[16];
  float proj_inv[16];
  float wv_inv[16];
  float width, height;
  // camera_ray's constants: the ray origin wv_inv * (0,0,0,1) (the same
  // float operations, done once), and 1/width, 1/height when those are powers
  // of two (x * 2^-k = x / 2^k exactly; 0 otherwise: divide)
  float ro[3];
  float inv_w, inv_h;
};

// A (mesh, instance) pair: where its vertices start in the flattened arrays.
// Blocks per job of the loss reduction (a power of two: the completion
// ticket counts modulo this and wraps around cleanly).
constexpr int kLossBlocks = 64;

struct BlockDev {
  int vert_off;   // first flattened vertex
  int tri_off;    // first flattened triangle
  int mesh;       // mesh id (geomId)
  int inst;       // instance id (instId)
};

// Per-mesh data used by shading and gradient scatter.
struct MeshDev {
  const float* tex;   // w*h*c texture or null
  int tex_w, tex_h, tex_c;
  int dslot;          // differentiable slot, -1 if the mesh is static
  int64_t g_base;     // offset of this mesh's DMesh block in the flat gradient
  int pos_off, color_off, tex_off, tr_off;
  int n_vertices, n_instances;
  int block0;         // flattened block of instance 0 (the instances' blocks follow it)
};

struct ModelParams {
  float light_pos[3];
  float light_intensity;
  float ambient;
  int path_depth;
  uint32_t seed;
};

// Light-space grid of the point light's shadow rays: a view from the light
// position toward the scene's bounding sphere.  A point q maps to grid
// coordinates (dot(q-L, u)/z * scale + half, dot(q-L, v)/z * scale + half)
// with z = dot(q-L, w); every point of the sphere has z > 0 and lands in
// [0, G) x [0, G).  ok = 0: the light is inside (or too close to) the
// sphere, and shadow rays are traced.
struct LightGrid {
  float lx, ly, lz;  // light position
  float ux, uy, uz, vx, vy, vz, wx, wy, wz;
  float scale, half;
  int G, ok;
  int valid;     // the cell lists hold the current geometry (cleared by every refit)
  int overflow;  // the lists did not fit their buffer
};

// One render job: a committed scene, its BVH, views and buffers.  All
// pointers are device pointers.
struct JobDev {
  // flattened prepared scene (Scene::prepare_for_render, scene_utils.cpp:98-173)
  int n_vertices;
  int n_tris;
  int n_blocks;
  int n_meshes;
  const float4* pos;     // world positions
  const float4* orig;    // untransformed positions
  const float4* col;
  const float4* nrm;
  const float4* tan;     // tangents (PATH_TEST only, else null)
  const float2* tc;
  const int4* tri_v;     // per flattened triangle: global ids A,B,C and block index
  const BlockDev* blocks;
  const MeshDev* meshes;
  const float* tr_inv0;  // inverse transforms of mesh 0 (16 per instance)
  const float* block_tr; // per block: transform (16, column-major), inverse transpose (16)
  // BVH: internal nodes (4 float4 each) and leaf triangles in leaf order
  const float4* nodes;
  const float4* tri;     // 3 float4 per leaf: (A, id bits), (e1), (e2)
  // 4-wide view of the same hierarchy (builds with -DDRGB_BVH4, which
  // traverse it instead of the binary nodes; measured slower on GB300 than
  // the binary traversal), 8 float4 per binary internal node p:
  // the boxes of p's children with every internal child replaced by its two
  // children (slots 0-1 from child 0, 2-3 from child 1), stored as lo_x[4],
  // hi_x[4], lo_y[4], hi_y[4], lo_z[4], hi_z[4], links[4] (int bits: >= 0
  // internal node, < 0 leaf ~k, kEmpty4 unused), one unused float4
  const float4* nodes4;
  int root;              // >= 0 internal node, < 0 leaf ~k, INT_MIN if empty
  int top_n;             // internal nodes 0..top_n-1 (the top levels, breadth-first numbering)
                         // are read from the block's shared copy; 0: none staged
  const int* leaf_of;    // flattened triangle -> its leaf slot in `tri`
  int trace_bruteforce;  // 1: test every triangle (reference loop order)
  int trace_limit;       // node pops per ray before the traversal gives up and raises ERR_TRAVERSAL_LIMIT
  // model
  int mode;
  int spp;               // requested spp (Hammersley count)
  int sq;                // floor(sqrt(spp))
  int S;                 // sq*sq samples per pixel
  const float* ham;      // 2*spp Hammersley offsets
  ModelParams mp;
  // views
  int n_views;
  const CamDev* cams;
  int W, H;              // view size (all views of a gradient call share it)
  // gradient buffer (DScene layout, all differentiable meshes concatenated)
  float* grad;
  uint32_t* err;
  // per-call I/O of the pixel kernel
  float* images;            // 3 floats per pixel (null: not written)
  const int64_t* img_off;   // first pixel of each view in images/targets
  const float* targets;     // 3 floats per pixel
  float4* adj;              // adjoint image, W*H per view
  const float* adj_in;      // caller-supplied adjoint images (d_render), 3 floats per pixel
  double* loss_part;        // one partial sum per pixel item of this job
  double* loss_blk;         // kLossBlocks chunk sums per view
  unsigned* loss_ticket;    // blocks of the loss reduction done (modulo kLossBlocks)
  float* loss_out;          // final loss of the last call
  int tile_w, tile_h;
  int item_base, item_count;  // pixel items of this job in the launch's item list
  // edge sampling (edge_derivatives, drender.h:235-425)
  const int4* edges;        // v0, v1 (global ids), vn0, vn1 (mesh-local ids)
  const int2* edge_mi;      // mesh, instance
  const int2* edge_tris;    // the two flattened triangles sharing the edge (-1: boundary edge)
  int edge_sil;             // 1: per view, only silhouette and boundary edges are sampled
  int n_edges;
  float4* proj;             // per view per vertex: pixel x, pixel y, world z
  float* pmf;               // per view n_edges
  float* cdf;               // per view n_edges + 1
  int4* queue;              // surviving samples: view, sample index, edge id
  int* queue_count;
  int queue_cap;
  int edge_samples;
  const float* rnd;         // 2 * edge_samples replayed random numbers
  const int* rnd_order;     // sample indices by increasing first random number (may be null)
  int edge_exact;           // 1: full 2x3 screen Jacobian through the instance's own transform
  uint32_t edge_key_base;   // first queue-sort key of this job in a batch
  // optional work counters (rays, box tests, triangle tests, footprint tests); null normally
  unsigned long long* work;
  // deterministic reduction: gradient contributions become records
  // {gradient index of 3 consecutive floats, value} in slots fixed by their
  // producer (work item / pass / lane, or view / edge sample), summed later
  // in a fixed order instead of by float atomics
  int det;
  int rec_item_cap;          // record slots of one pixel work item
  uint32_t* rec_key;
  float4* rec_val;
  int* rec_count;            // records per region: work items, then (view, sample) edge regions
  float* det_tr;             // deterministic mode with one transform block: 12 floats per edge sample
  int det_tr_key;            // (view, sample order), summed in a fixed order into grad[det_tr_key + 0..11]
  // stored adjoint hits (one float4 {t, u, v, triangle} per adjoint sample)
  float4* hit_buf;
  // rasterised primary visibility: per forward / adjoint sample the nearest
  // hit found by the raster pass, {t, u, v, triangle bits} (triangle -1: no
  // hit); null: the samples are traced through the hierarchy
  float4* vis_fwd;
  float4* vis_adj;
  // point-light model: u, v of the hit per forward / adjoint sample, and the
  // float4 record holds the shading point ro + rd * (t - 1e-5) in place of
  // t (what the model uses of the ray; the pixel kernel then builds no ray)
  float2* vis_uv_fwd;
  float2* vis_uv_adj;
  const uint32_t* ra_state;  // bit 0: the raster pass wrote nothing this call; bit 1: its tile lists
                             // hold the current geometry (cleared by every refit)
  // the raster pass's screen tiles (tw x th pixels, ntx x nty per view): per
  // (view, tile) the list offsets ([count] = total), the (view, leaf) entries
  // and their footprints (4 float4 each); null when there is no raster pass
  const uint32_t* ra_tiles;
  const int* ra_list;
  const float4* ra_rec;
  int ra_tw, ra_th, ra_ntx, ra_nty;
  // point-light shadow rays through light-space cells (null: traced)
  const LightGrid* sh_grid;
  const uint32_t* sh_cells;  // per cell the offset of its list, [G*G] = total
  const int* sh_list;        // triangle leaf slots
  const float4* sh_rec;      // per leaf slot its light-space footprint (box, three edge lines)
};

// Record slots a work item of NS samples may fill (deterministic mode):
// per pass of 32 samples, 3 per lane for vertex colours, 4 for texture taps.
__host__ __device__ inline int item_record_cap(int mode, int NS) {
  const int passes = (NS + 31) / 32;
  return passes * 32 * (model_has_tex(mode) ? 4 : 3);
}

// Partial sum of one gradient index in the deterministic reduction.
constexpr uint32_t kNoKey = 0xFFFFFFFFu;
struct DetFrag {
  uint32_t key;  // kNoKey: empty
  float x, y, z;
};

// Record slots of the edge region of sample i of a view.
constexpr int kEdgeRecords = 6;  // two vertex positions, four rows of the instance matrix
__device__ __forceinline__ int64_t edge_region(const JobDev& J, int view, int i) {
  return (int64_t)J.item_count + (int64_t)view * J.edge_samples + i;
}
__device__ __forceinline__ int64_t edge_rec_slot(const JobDev& J, int view, int i) {
  return (int64_t)J.item_count * J.rec_item_cap + ((int64_t)view * J.edge_samples + i) * kEdgeRecords;
}

// Source arrays of one mesh read by the flattening kernel.
struct MeshSrc {
  const float* v;
  const float* col;
  const float* nrm;
  const float* tc;
  const float* tan;
};

// One differentiable mesh as the optimiser updates it.
struct OptMesh {
  int64_t base;
  int full;
  int pos_off, color_off, tex_off, tr_off;
  int nv, n_inst;
  float* vertices;
  float* colors;
  float* texture;
  float* transforms;
  float* rparams;  // restricted mesh: 7 parameters per instance at tr_off (else null)
};

constexpr int kBatchMaxDMeshes = 4;

// Everything the per-iteration maintenance passes of one job touch (scene
// flattening, LBVH refit, optimiser), for launches that cover many jobs.
struct JobAux {
  int n_vertices, n_tris, n_blocks;
  const int* vblock;
  const BlockDev* blocks;
  const MeshSrc* src;
  const float* const* tr_tab;
  float* block_tr;
  float4 *pos, *orig, *col, *nrm, *tan;
  float2* tc;
  const int4* tri_v;
  const int* perm;
  int* leaf_of;
  float4* tri;
  float4* nodes;
  float4* nodes4;
  const int* leaf_parent;
  const int* node_parent;
  int* counters;
  float* grad;
  int64_t grad_total;
  float *m, *G, *lr;
  int* iter;
  float* losses;
  int losses_cap;
  const float* loss_out;
  int alg, flags, mode, decay_period;
  float decay_mult;
  int n_dmesh;
  OptMesh dm[kBatchMaxDMeshes];
};

// A contiguous run of work of one job (and one view or sub-range): global
// chunk indices [begin, begin + ceil(count / chunk)) map to it.
struct Seg {
  int job;
  int sub;
  int begin;
  int count;
};

// Segment of a global chunk index (segments sorted by begin).
__device__ __forceinline__ int find_seg(const Seg* segs, int n, int chunk) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&segs[mid].begin) <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Exact float3 helpers (LiteMath operation order).
// ---------------------------------------------------------------------------
struct f3 {
  float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float length(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ f3 normalize(f3 a) {
  float inv = 1.0f / length(a);
  return a * inv;
}
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
  float dx = a.x * b.y - a.y * b.x;
  float dy = a.y * b.z - a.z * b.y;
  float dz = a.z * b.x - a.x * b.z;
  return mk(dy, dz, dx);
}
__device__ __forceinline__ float ref_sign(float x) { return x == 0.0f ? 0.0f : (x < 0.0f ? -1.0f : 1.0f); }
__device__ __forceinline__ float ref_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float ref_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float ref_clamp(float u, float a, float b) { return ref_min(ref_max(a, u), b); }
__device__ __forceinline__ int clampi(int u, int a, int b) {
  int m = (a < u) ? u : a;
  return (b < m) ? b : m;
}
__device__ __forceinline__ f3 ld3(const float4* p, int i) {
  float4 v = __ldg(p + i);
  return mk(v.x, v.y, v.z);
}
__device__ __forceinline__ f3 f4to3(float4 v) { return mk(v.x, v.y, v.z); }

// mat4_colmajor_mul_vec4 with w = 1 (LiteMath.h:1342-1348, 1451-1457)
__device__ __forceinline__ f3 mat_pt(const float* m, f3 p) {
  return mk(p.x * m[0] + p.y * m[4] + p.z * m[8] + 1.0f * m[12], p.x * m[1] + p.y * m[5] + p.z * m[9] + 1.0f * m[13],
            p.x * m[2] + p.y * m[6] + p.z * m[10] + 1.0f * m[14]);
}

// Barycentric interpolation a*(1-u-v) + b*v + u*c (shade_simple.cpp:36).
__device__ __forceinline__ f3 interp(f3 a, f3 b, f3 c, float u, float v) {
  const float w0 = 1.0f - u - v;
  return (a * w0 + b * v) + c * u;
}

// ---------------------------------------------------------------------------
// 4x4 inverse with the cofactor pairing of LiteMath.h:1551-1633 (column-major
// storage, element (r,c) at m[4c+r]).  Used on the host for camera inverses
// and on the device for the normal transform.
// ---------------------------------------------------------------------------
#define MM(m, r, c) ((m)[4 * (c) + (r)])
__host__ __device__ inline void mat_inverse44(const float* m1, float* out) {
  float tmp[12], m[16];
  tmp[0] = MM(m1, 2, 2) * MM(m1, 3, 3);
  tmp[1] = MM(m1, 2, 3) * MM(m1, 3, 2);
  tmp[2] = MM(m1, 2, 1) * MM(m1, 3, 3);
  tmp[3] = MM(m1, 2, 3) * MM(m1, 3, 1);
  tmp[4] = MM(m1, 2, 1) * MM(m1, 3, 2);
  tmp[5] = MM(m1, 2, 2) * MM(m1, 3, 1);
  tmp[6] = MM(m1, 2, 0) * MM(m1, 3, 3);
  tmp[7] = MM(m1, 2, 3) * MM(m1, 3, 0);
  tmp[8] = MM(m1, 2, 0) * MM(m1, 3, 2);
  tmp[9] = MM(m1, 2, 2) * MM(m1, 3, 0);
  tmp[10] = MM(m1, 2, 0) * MM(m1, 3, 1);
  tmp[11] = MM(m1, 2, 1) * MM(m1, 3, 0);
  MM(m, 0, 0) = tmp[0] * MM(m1, 1, 1) + tmp[3] * MM(m1, 1, 2) + tmp[4] * MM(m1, 1, 3);
  MM(m, 0, 0) -= tmp[1] * MM(m1, 1, 1) + tmp[2] * MM(m1, 1, 2) + tmp[5] * MM(m1, 1, 3);
  MM(m, 1, 0) = tmp[1] * MM(m1, 1, 0) + tmp[6] * MM(m1, 1, 2) + tmp[9] * MM(m1, 1, 3);
  MM(m, 1, 0) -= tmp[0] * MM(m1, 1, 0) + tmp[7] * MM(m1, 1, 2) + tmp[8] * MM(m1, 1, 3);
  MM(m, 2, 0) = tmp[2] * MM(m1, 1, 0) + tmp[7] * MM(m1, 1, 1) + tmp[10] * MM(m1, 1, 3);
  MM(m, 2, 0) -= tmp[3] * MM(m1, 1, 0) + tmp[6] * MM(m1, 1, 1) + tmp[11] * MM(m1, 1, 3);
  MM(m, 3, 0) = tmp[5] * MM(m1, 1, 0) + tmp[8] * MM(m1, 1, 1) + tmp[11] * MM(m1, 1, 2);
  MM(m, 3, 0) -= tmp[4] * MM(m1, 1, 0) + tmp[9] * MM(m1, 1, 1) + tmp[10] * MM(m1, 1, 2);
  MM(m, 0, 1) = tmp[1] * MM(m1, 0, 1) + tmp[2] * MM(m1, 0, 2) + tmp[5] * MM(m1, 0, 3);
  MM(m, 0, 1) -= tmp[0] * MM(m1, 0, 1) + tmp[3] * MM(m1, 0, 2) + tmp[4] * MM(m1, 0, 3);
  MM(m, 1, 1) = tmp[0] * MM(m1, 0, 0) + tmp[7] * MM(m1, 0, 2) + tmp[8] * MM(m1, 0, 3);
  MM(m, 1, 1) -= tmp[1] * MM(m1, 0, 0) + tmp[6] * MM(m1, 0, 2) + tmp[9] * MM(m1, 0, 3);
  MM(m, 2, 1) = tmp[3] * MM(m1, 0, 0) + tmp[6] * MM(m1, 0, 1) + tmp[11] * MM(m1, 0, 3);
  MM(m, 2, 1) -= tmp[2] * MM(m1, 0, 0) + tmp[7] * MM(m1, 0, 1) + tmp[10] * MM(m1, 0, 3);
  MM(m, 3, 1) = tmp[4] * MM(m1, 0, 0) + tmp[9] * MM(m1, 0, 1) + tmp[10] * MM(m1, 0, 2);
  MM(m, 3, 1) -= tmp[5] * MM(m1, 0, 0) + tmp[8] * MM(m1, 0, 1) + tmp[11] * MM(m1, 0, 2);
  tmp[0] = MM(m1, 0, 2) * MM(m1, 1, 3);
  tmp[1] = MM(m1, 0, 3) * MM(m1, 1, 2);
  tmp[2] = MM(m1, 0, 1) * MM(m1, 1, 3);
  tmp[3] = MM(m1, 0, 3) * MM(m1, 1, 1);
  tmp[4] = MM(m1, 0, 1) * MM(m1, 1, 2);
  tmp[5] = MM(m1, 0, 2) * MM(m1, 1, 1);
  tmp[6] = MM(m1, 0, 0) * MM(m1, 1, 3);
  tmp[7] = MM(m1, 0, 3) * MM(m1, 1, 0);
  tmp[8] = MM(m1, 0, 0) * MM(m1, 1, 2);
  tmp[9] = MM(m1, 0, 2) * MM(m1, 1, 0);
  tmp[10] = MM(m1, 0, 0) * MM(m1, 1, 1);
  tmp[11] = MM(m1, 0, 1) * MM(m1, 1, 0);
  MM(m, 0, 2) = tmp[0] * MM(m1, 3, 1) + tmp[3] * MM(m1, 3, 2) + tmp[4] * MM(m1, 3, 3);
  MM(m, 0, 2) -= tmp[1] * MM(m1, 3, 1) + tmp[2] * MM(m1, 3, 2) + tmp[5] * MM(m1, 3, 3);
  MM(m, 1, 2) = tmp[1] * MM(m1, 3, 0) + tmp[6] * MM(m1, 3, 2) + tmp[9] * MM(m1, 3, 3);
  MM(m, 1, 2) -= tmp[0] * MM(m1, 3, 0) + tmp[7] * MM(m1, 3, 2) + tmp[8] * MM(m1, 3, 3);
  MM(m, 2, 2) = tmp[2] * MM(m1, 3, 0) + tmp[7] * MM(m1, 3, 1) + tmp[10] * MM(m1, 3, 3);
  MM(m, 2, 2) -= tmp[3] * MM(m1, 3, 0) + tmp[6] * MM(m1, 3, 1) + tmp[11] * MM(m1, 3, 3);
  MM(m, 3, 2) = tmp[5] * MM(m1, 3, 0) + tmp[8] * MM(m1, 3, 1) + tmp[11] * MM(m1, 3, 2);
  MM(m, 3, 2) -= tmp[4] * MM(m1, 3, 0) + tmp[9] * MM(m1, 3, 1) + tmp[10] * MM(m1, 3, 2);
  MM(m, 0, 3) = tmp[2] * MM(m1, 2, 2) + tmp[5] * MM(m1, 2, 3) + tmp[1] * MM(m1, 2, 1);
  MM(m, 0, 3) -= tmp[4] * MM(m1, 2, 3) + tmp[0] * MM(m1, 2, 1) + tmp[3] * MM(m1, 2, 2);
  MM(m, 1, 3) = tmp[8] * MM(m1, 2, 3) + tmp[0] * MM(m1, 2, 0) + tmp[7] * MM(m1, 2, 2);
  MM(m, 1, 3) -= tmp[6] * MM(m1, 2, 2) + tmp[9] * MM(m1, 2, 3) + tmp[1] * MM(m1, 2, 0);
  MM(m, 2, 3) = tmp[6] * MM(m1, 2, 1) + tmp[11] * MM(m1, 2, 3) + tmp[3] * MM(m1, 2, 0);
  MM(m, 2, 3) -= tmp[10] * MM(m1, 2, 3) + tmp[2] * MM(m1, 2, 0) + tmp[7] * MM(m1, 2, 1);
  MM(m, 3, 3) = tmp[10] * MM(m1, 2, 2) + tmp[4] * MM(m1, 2, 0) + tmp[9] * MM(m1, 2, 1);
  MM(m, 3, 3) -= tmp[8] * MM(m1, 2, 1) + tmp[11] * MM(m1, 2, 2) + tmp[5] * MM(m1, 2, 0);
  const float k = 1.0f / (MM(m1, 0, 0) * MM(m, 0, 0) + MM(m1, 0, 1) * MM(m, 1, 0) + MM(m1, 0, 2) * MM(m, 2, 0) +
                          MM(m1, 0, 3) * MM(m, 3, 0));
  for (int i = 0; i < 16; i++) out[i] = m[i] * k;
}

#undef MM

// ---------------------------------------------------------------------------
// Camera rays: EyeRayDirNormalized + transform_ray3f (raytrace.h:49-76) as
// used by BruteForce3D::CastSingleRay (raytrace3d_bf.cpp:158-174).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void camera_ray(const CamDev& c, float x, float y, f3& ro, f3& rd) {
  const float xn = c.inv_w != 0.0f ? x * c.inv_w : x / c.width;
  const float yn = c.inv_h != 0.0f ? y * c.inv_h : y / c.height;
  const float V0 = 2.0f * xn - 1.0f, V1 = -2.0f * yn + 1.0f, V2 = 0.0f, V3 = 1.0f;
  const float* B = c.proj_inv;
  float r0 = V0 * B[0] + V1 * B[4] + V2 * B[8] + V3 * B[12];
  float r1 = V0 * B[1] + V1 * B[5] + V2 * B[9] + V3 * B[13];
  float r2 = V0 * B[2] + V1 * B[6] + V2 * B[10] + V3 * B[14];
  float r3 = V0 * B[3] + V1 * B[7] + V2 * B[11] + V3 * B[15];
  r0 /= r3;
  r1 /= r3;
  r2 /= r3;
  const f3 dir = normalize(mk(r0, r1, r2));
  const f3 p0 = mk(0.0f, 0.0f, 0.0f);
  const f3 pos = mk(c.ro[0], c.ro[1], c.ro[2]);  // mat_pt(c.wv_inv, p0)
  const f3 pos2 = mat_pt(c.wv_inv, p0 + dir * 100.0f);
  ro = pos;
  rd = normalize(pos2 - pos);
}

// ---------------------------------------------------------------------------
// Ray/triangle test in the operation order of raytrace3d_bf.cpp:127-140.
// Returns true when the brute-force caster would accept the hit for the
// current best distance; u, v, t are bit-identical to the caster's.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool mt_test(f3 pos, f3 dir, f3 A, f3 edge1, f3 edge2, float tNear, float& t, float& u,
                                        float& v) {
  const f3 pvec = cross(dir, edge2);
  const f3 tvec = pos - A;
  const float e1dpv = dot(edge1, pvec);
  const float signv = ref_sign(e1dpv);
  const float invDet = signv / ref_max(signv * e1dpv, 1e-6f);
  v = dot(tvec, pvec) * invDet;
  if (!(v > 0.0f)) return false;
  const f3 qvec = cross(tvec, edge1);
  u = dot(qvec, dir) * invDet;
  if (!(u > 0.0f) || !(u + v < 1.0f)) return false;
  t = dot(edge2, qvec) * invDet;
  return t > tNear;
}

struct Hit {
  float t, u, v;
  int tri;  // flattened triangle index, -1 = miss
};

// Three-input min / max (one instruction on sm_100 and later); exact, so the
// grouping does not change any result.
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000 && !defined(DRGB_NO_MINMAX3)
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
#else
  return fminf(fminf(a, b), c);
#endif
}
__device__ __forceinline__ float fmax3f(float a, float b, float c) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000 && !defined(DRGB_NO_MINMAX3)
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
#else
  return fmaxf(fmaxf(a, b), c);
#endif
}

// Ray/box slab test with precomputed inverse direction; returns the entry
// distance (or +inf when the box is missed within [lo_t, hi_t]).
__device__ __forceinline__ float slab(float lx, float hx, float ly, float hy, float lz, float hz, f3 inv, f3 oi,
                                      float lo_t, float hi_t) {
  const float tx0 = __fmaf_rn(lx, inv.x, -oi.x), tx1 = __fmaf_rn(hx, inv.x, -oi.x);
  const float ty0 = __fmaf_rn(ly, inv.y, -oi.y), ty1 = __fmaf_rn(hy, inv.y, -oi.y);
  const float tz0 = __fmaf_rn(lz, inv.z, -oi.z), tz1 = __fmaf_rn(hz, inv.z, -oi.z);
  const float tmin = fmax3f(fminf(tx0, tx1), fminf(ty0, ty1), fmaxf(fminf(tz0, tz1), lo_t));
  const float tmax = fmin3f(fmaxf(tx0, tx1), fmaxf(ty0, ty1), fminf(fmaxf(tz0, tz1), hi_t));
  return tmin <= tmax ? tmin : __int_as_float(0x7f800000);
}

// The same test with each axis's two planes as one packed pair (FFMA2:
// two FP32 FMAs in one instruction on sm_100 and later; each lane rounds
// as __fmaf_rn, so the result is the scalar test's).  x, y, z: (lo, hi) of
// one axis, adjacent in the node layout; i*, o*: the inverse direction and
// -origin*inverse, duplicated in both lanes.
__device__ __forceinline__ float slab_p(float2 x, float2 y, float2 z, float2 ix, float2 iy, float2 iz, float2 ox,
                                        float2 oy, float2 oz, float lo_t, float hi_t) {
  const float2 tx = __ffma2_rn(x, ix, ox), ty = __ffma2_rn(y, iy, oy), tz = __ffma2_rn(z, iz, oz);
  const float tmin = fmax3f(fminf(tx.x, tx.y), fminf(ty.x, ty.y), fmaxf(fminf(tz.x, tz.y), lo_t));
  const float tmax = fmin3f(fmaxf(tx.x, tx.y), fmaxf(ty.x, ty.y), fminf(fmaxf(tz.x, tz.y), hi_t));
  return tmin <= tmax ? tmin : __int_as_float(0x7f800000);
}

__device__ __forceinline__ float safe_inv(float d) {
  const float eps = 1e-20f;
  if (fabsf(d) < eps) d = copysignf(eps, d);
  return 1.0f / d;
}

// Slack on the culling distance so that no box whose triangle the
// brute-force test would accept is skipped (boxes are also padded).
__device__ __forceinline__ float cull_bound(float t) { return t + fabsf(t) * 4e-6f + 1e-6f; }

// -DDRGB_TOP_SMEM: the top levels of the hierarchy in shared memory.  Kernels
// that trace for a single job copy the first top_n internal nodes there once
// per block (stage_top_nodes) before their first traversal; every other
// kernel traces with top_n = 0.  127 nodes = the top 7 levels of the
// breadth-first numbered top of the binned-SAH hierarchy, 8 KB.  Off by
// default: the icosphere workload ran 9 % slower with it on GB300 (a branch
// on every node visit and the staging, for nodes that are L1 hits anyway;
// the pixel kernel's L1 hit rate fell from 79 % to 64 % as those hits left
// L1).  A smaller shared footprint alone changed nothing.
constexpr int kTopNodes = 127;
#ifdef DRGB_TOP_SMEM
static __shared__ float4 g_top_nodes[4 * kTopNodes];

__device__ __forceinline__ void stage_top_nodes(const JobDev& J) {
  for (int i = threadIdx.x; i < 4 * J.top_n; i += blockDim.x) g_top_nodes[i] = __ldg(J.nodes + i);
  __syncthreads();
}
#else
__device__ __forceinline__ void stage_top_nodes(const JobDev&) {}
#endif

// Nearest hit (ANY=false) or any hit (ANY=true) in [tNear, tFar).  Equal
// distances resolve to the lowest flattened triangle index, which is the
// triangle the reference's in-order brute-force loop keeps.
__device__ __forceinline__ void add_work(const JobDev& J, unsigned boxes, unsigned tris) {
  if (J.work) {
    atomicAdd(J.work + 0, 1ull);
    atomicAdd(J.work + 1, (unsigned long long)boxes);
    atomicAdd(J.work + 2, (unsigned long long)tris);
  }
}

// Work of a ray resolved against a screen-tile or light-cell list: `fp`
// footprint (box and edge-line) tests, `tris` ray/triangle tests; `ray`: it
// counts as a ray (a camera ray built for it).
__device__ __forceinline__ void add_list_work(const JobDev& J, bool ray, unsigned fp, unsigned tris) {
  if (J.work) {
    if (ray) atomicAdd(J.work + 0, 1ull);
    if (tris) atomicAdd(J.work + 2, (unsigned long long)tris);
    if (fp) atomicAdd(J.work + 3, (unsigned long long)fp);
  }
}

// Traversal is kept out of line by default: it is called from several
// places per kernel (camera hits, shadow rays, re-traced adjoint samples),
// and one shared copy of the loop keeps the kernels' code within the
// instruction cache.  Build with -DDRGB_TRACE_INLINE to inline it instead.
#ifdef DRGB_TRACE_INLINE
#define DRGB_TRACE_ATTR __forceinline__
#else
#define DRGB_TRACE_ATTR __noinline__
#endif
#ifndef DRGB_TRACE_SPLIT
// One out-of-line traversal for nearest and any hits (the any-hit exit is a
// run-time test): half the traversal code in every kernel, fewer
// instruction-fetch stalls (+10 % on the point-light workload on GB300;
// -DDRGB_TRACE_SPLIT builds one copy per kind).
static __device__ DRGB_TRACE_ATTR bool trace_impl(const JobDev& J, f3 o, f3 d, float tNear, float tFar,
                                                  Hit& best, const bool ANY, const int seed);
template <bool ANY>
__device__ __forceinline__ bool trace(const JobDev& J, f3 o, f3 d, float tNear, float tFar, Hit& best,
                                      int seed = -1) {
  return trace_impl(J, o, d, tNear, tFar, best, ANY, seed);
}
static __device__ DRGB_TRACE_ATTR bool trace_impl(const JobDev& J, f3 o, f3 d, float tNear, float tFar,
                                                  Hit& best, const bool ANY, const int seed) {
#else
template <bool ANY>
__device__ DRGB_TRACE_ATTR bool trace(const JobDev& J, f3 o, f3 d, float tNear, float tFar, Hit& best,
                                      int seed = -1) {
#endif
  best.t = tFar;
  best.tri = -1;
  best.u = 0.0f;
  best.v = 0.0f;
  if (J.n_tris <= 0) return false;
  unsigned n_box = 0, n_tri = 0;
  if (J.trace_bruteforce) {
    for (int k = 0; k < J.n_tris; k++) {
      const float4 a = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
      const int id = __float_as_int(a.w);
      float t, u, v;
      if (mt_test(o, d, f4to3(a), f4to3(e1), f4to3(e2), tNear, t, u, v)) {
        if (t < best.t || (t == best.t && id < best.tri)) {
          best.t = t;
          best.u = u;
          best.v = v;
          best.tri = id;
          if (ANY) {
            add_work(J, 0, k + 1);
            return true;
          }
        }
      }
    }
    add_work(J, 0, J.n_tris);
    return best.tri >= 0;
  }
  // seed: a triangle likely to be the nearest hit (the hit of a nearby ray),
  // tested first so that the traversal culls with its distance from the
  // start.  A valid candidate cannot change the result (the same test and
  // tie rule decide, and the culling keeps a slack).
  if (!ANY && seed >= 0 && J.leaf_of) {
    const int k = __ldg(J.leaf_of + seed);
    const float4 a = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
    float t, u, v;
    if (mt_test(o, d, f4to3(a), f4to3(e1), f4to3(e2), tNear, t, u, v) && t < best.t) {
      best.t = t;
      best.u = u;
      best.v = v;
      best.tri = __float_as_int(a.w);
    }
  }
  const f3 inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
  const f3 oi = mk(o.x * inv.x, o.y * inv.y, o.z * inv.z);
  const float lo_t = tNear - fabsf(tNear) * 4e-6f - 1e-6f;
#ifndef DRGB_BVH4
  const float2 ix = make_float2(inv.x, inv.x), iy = make_float2(inv.y, inv.y), iz = make_float2(inv.z, inv.z);
  const float2 ox = make_float2(-oi.x, -oi.x), oy = make_float2(-oi.y, -oi.y), oz = make_float2(-oi.z, -oi.z);
#endif
#ifdef DRGB_SMEM_STACK
  // the top DRGB_SMEM_STACK entries in shared memory (one column per thread,
  // blocks of at most 256 threads), deeper ones in local memory
  __shared__ int s_stack[DRGB_SMEM_STACK * 256];
  int* const sst = s_stack + threadIdx.x;
  int stack[kStackSize - DRGB_SMEM_STACK];
#define DRGB_PUSH(v) (sp < DRGB_SMEM_STACK ? (sst[256 * sp] = (v)) : (stack[sp - DRGB_SMEM_STACK] = (v))), sp++
#define DRGB_POP() (--sp, sp < DRGB_SMEM_STACK ? sst[256 * sp] : stack[sp - DRGB_SMEM_STACK])
#else
  int stack[kStackSize];
#define DRGB_PUSH(v) stack[sp++] = (v)
#define DRGB_POP() stack[--sp]
#endif
  int sp = 0;
  int node = J.root;
  int guard = 0;
  float hi_t = cull_bound(best.t);  // renewed when best.t shrinks
  while (true) {
    if (node >= 0) {
#ifndef DRGB_BVH4
      float4 n0, n1, n2, n3;
#ifdef DRGB_TOP_SMEM
      if (node < J.top_n) {
        n0 = g_top_nodes[4 * node + 0];
        n1 = g_top_nodes[4 * node + 1];
        n2 = g_top_nodes[4 * node + 2];
        n3 = g_top_nodes[4 * node + 3];
      } else
#endif
      {
        n0 = __ldg(J.nodes + 4 * node + 0);
        n1 = __ldg(J.nodes + 4 * node + 1);
        n2 = __ldg(J.nodes + 4 * node + 2);
        n3 = __ldg(J.nodes + 4 * node + 3);
      }
      n_box += 2;
      // packed (FFMA2) slab tests: 6 instructions for the 12 plane distances
      // (GB300: -4 % instructions and +1.5 % iterations/s on the point-light
      // and path workloads against the scalar slab())
      const float t0 = slab_p(make_float2(n0.x, n0.y), make_float2(n0.z, n0.w), make_float2(n2.x, n2.y), ix, iy, iz,
                              ox, oy, oz, lo_t, hi_t);
      const float t1 = slab_p(make_float2(n1.x, n1.y), make_float2(n1.z, n1.w), make_float2(n2.z, n2.w), ix, iy, iz,
                              ox, oy, oz, lo_t, hi_t);
      const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      const bool h0 = t0 <= hi_t, h1 = t1 <= hi_t;
      if (h0 && h1) {
        const bool first0 = t0 <= t1;
        if (sp >= kStackSize) {
          atomicOr(J.err, ERR_STACK_OVERFLOW);
          add_work(J, n_box, n_tri);
          return best.tri >= 0;
        }
        DRGB_PUSH(first0 ? c1 : c0);
        node = first0 ? c0 : c1;
        continue;
      } else if (h0) {
        node = c0;
        continue;
      } else if (h1) {
        node = c1;
        continue;
      }
#else
      const float4* q = J.nodes4 + 8 * node;
      const float4 LX = __ldg(q + 0), HX = __ldg(q + 1), LY = __ldg(q + 2), HY = __ldg(q + 3);
      const float4 LZ = __ldg(q + 4), HZ = __ldg(q + 5), LK = __ldg(q + 6);
      n_box += 4;
      const float inf = __int_as_float(0x7f800000);
      int c0 = __float_as_int(LK.x), c1 = __float_as_int(LK.y), c2 = __float_as_int(LK.z), c3 = __float_as_int(LK.w);
      float t0 = c0 == kEmpty4 ? inf : slab(LX.x, HX.x, LY.x, HY.x, LZ.x, HZ.x, inv, oi, lo_t, hi_t);
      float t1 = c1 == kEmpty4 ? inf : slab(LX.y, HX.y, LY.y, HY.y, LZ.y, HZ.y, inv, oi, lo_t, hi_t);
      float t2 = c2 == kEmpty4 ? inf : slab(LX.z, HX.z, LY.z, HY.z, LZ.z, HZ.z, inv, oi, lo_t, hi_t);
      float t3 = c3 == kEmpty4 ? inf : slab(LX.w, HX.w, LY.w, HY.w, LZ.w, HZ.w, inv, oi, lo_t, hi_t);
      // nearest first: a 4-input sorting network on (t, link)
#define DRGB_CSWAP(ta, ca, tb, cb)                 \
  if (tb < ta) {                                  \
    const float tt = ta; ta = tb; tb = tt;        \
    const int cc = ca; ca = cb; cb = cc;          \
  }
      DRGB_CSWAP(t0, c0, t1, c1);
      DRGB_CSWAP(t2, c2, t3, c3);
      DRGB_CSWAP(t0, c0, t2, c2);
      DRGB_CSWAP(t1, c1, t3, c3);
      DRGB_CSWAP(t1, c1, t2, c2);
#undef DRGB_CSWAP
      if (t0 <= hi_t) {
        if (sp + 3 > kStackSize) {
          atomicOr(J.err, ERR_STACK_OVERFLOW);
          add_work(J, n_box, n_tri);
          return best.tri >= 0;
        }
        if (t3 <= hi_t) DRGB_PUSH(c3);
        if (t2 <= hi_t) DRGB_PUSH(c2);
        if (t1 <= hi_t) DRGB_PUSH(c1);
        node = c0;
        continue;
      }
#endif
    } else {
      const int k = ~node;
      const float4 a = __ldg(J.tri + 3 * k), e1 = __ldg(J.tri + 3 * k + 1), e2 = __ldg(J.tri + 3 * k + 2);
      const int id = __float_as_int(a.w);
      float t, u, v;
      n_tri++;
      if (mt_test(o, d, f4to3(a), f4to3(e1), f4to3(e2), tNear, t, u, v)) {
        if (t < best.t || (t == best.t && id < best.tri)) {
          best.t = t;
          best.u = u;
          best.v = v;
          best.tri = id;
          if (ANY) {
            add_work(J, n_box, n_tri);
            return true;
          }
          hi_t = cull_bound(best.t);
        }
      }
    }
    if (sp == 0) break;
    node = DRGB_POP();
    if (++guard > J.trace_limit) {
      atomicOr(J.err, ERR_TRAVERSAL_LIMIT);
      break;
    }
  }
  add_work(J, n_box, n_tri);
  return best.tri >= 0;
}
#undef DRGB_PUSH
#undef DRGB_POP

}  // namespace drgb

#include "shading.cuh"

namespace drgb {

// VertexShader (functions.h:5-13): pixel x,y of a world point.
__device__ __forceinline__ void vertex_shader(const CamDev& c, float vx, float vy, float vz, float& ox, float& oy) {
  const float* m = c.wvp;
  const float W = vx * m[3] + vy * m[7] + vz * m[11] + m[15];
  const float xNDC = (vx * m[0] + vy * m[4] + vz * m[8] + m[12]) / W;
  const float yNDC = -(vx * m[1] + vy * m[5] + vz * m[9] + m[13]) / W;
  ox = (xNDC * 0.5f + 0.5f) * c.width;
  oy = (yNDC * 0.5f + 0.5f) * c.height;
}

// VS_X_grad / VS_Y_grad (functions.cpp:21-163), same evaluation order.
__device__ __forceinline__ f3 vs_grad(const CamDev& c, f3 V, bool y) {
  const float* m = c.wvp;
  const float t1 = V.x, t0 = m[3], t3 = V.y, t2 = m[7], t5 = V.z, t4 = m[11];
  const float W = t1 * t0 + t3 * t2 + t5 * t4 + m[15];
  const float t7 = y ? m[1] : m[0];
  const float t9 = y ? m[5] : m[4];
  const float t11 = y ? m[9] : m[8];
  const float t13r = V.x * t7 + V.y * t9 + V.z * t11 + (y ? m[13] : m[12]);
  const float t13 = y ? -t13r : t13r;
  const float t6 = W;
  const float t14 = y ? c.height : c.width;
  const float d_xNDC = (1 * t14) * 0.5f;
  const float r6 = d_xNDC / t6;
  const float s6 = y ? -r6 : r6;
  const float d_W = d_xNDC * -t13 / (t6 * t6);
  return mk(s6 * t7 + d_W * t0, s6 * t9 + d_W * t2, s6 * t11 + d_W * t4);
}

}  // namespace drgb
