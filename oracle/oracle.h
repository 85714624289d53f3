/* CPU oracle for the differentiable mesh renderer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * renderer's CPU algorithm (FROL256/diffrender_tutorials, brute-force caster
 * build) used as the checker for the CUDA path and as the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
 * load it.  The product library never links or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks every entry point
 * below against fixtures produced by the reference itself
 * (tests/golden/make_golden.py, built by oracle/ref/build_ref.py).
 *
 * Arithmetic follows the reference operation by operation (no FMA
 * contraction: build with -ffp-contract=off), and gradient accumulation
 * replays the reference's 14-thread OpenMP static partition so that sums
 * are associated exactly as the reference associates them.
 */
#ifndef DRGB_ORACLE_H
#define DRGB_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Shading models; numbering of SHADING_MODEL (src/dmesh.h:16-23) plus two
 * models that have no reference counterpart. */
enum {
  ORC_SILHOUETTE = 1,
  ORC_VERTEX_COLOR = 2,
  ORC_TEXTURE_COLOR = 3,
  ORC_LAMBERT = 4,
  ORC_PHONG = 5,
  ORC_GGX = 6,
  ORC_PATH_TEST = 7,             /* shade_path_test.cpp:183-289, counter RNG in place of rand() */
  ORC_LAMBERT_POINT_VCOLOR = 16, /* point light + per-vertex albedo */
  ORC_PATH_DIFFUSE = 17          /* fixed-depth diffuse path tracer, counter RNG */
};

/* One mesh with its instances (TriangleMesh + transforms, common_src/scene.h:40-70,130-138). */
typedef struct orc_mesh {
  int32_t n_vertices;
  int32_t n_indices;
  const float* vertices;
  const float* colors;   /* may be NULL */
  const float* tc;       /* may be NULL */
  const float* normals;  /* may be NULL */
  const float* tangents; /* may be NULL */
  const uint32_t* indices;
  int32_t n_instances;
  const float* transforms; /* 16 floats per instance, column-major; NULL = identity */
  int32_t tex_w, tex_h, tex_channels;
  const float* texture; /* may be NULL */
  /* RESTRICTED_TRANSFORM mesh (scene.h:91-116,140-148): 7 floats per
   * instance {translate xyz, rotate xyz (radians), scale}; the matrices are
   * TransformR::to_mat of these and `transforms` is ignored.  NULL otherwise. */
  const float* restricted;
} orc_mesh;

/* Camera: 82 floats = world_view[16] proj[16] wvp[16] proj_inv[16] wv_inv[16] width height. */
#define ORC_CAM_FLOATS 82

/* Per-model constants of the two models without a reference counterpart. */
typedef struct orc_model_params {
  float light_pos[3];
  float light_intensity;
  float ambient;
  int32_t path_depth; /* bounces after the primary hit */
  uint32_t seed;
  /* edge-term chain rule: 0 the reference's edge_grad (drender.cpp:31-87),
   * 1 the full 2x3 screen Jacobian through the instance's own transform */
  int32_t edge_jacobian;
  /* edges the boundary term samples: 0 every edge (the reference), 1 only
   * silhouette and boundary edges of each view */
  int32_t edge_set;
} orc_model_params;

void orc_default_model_params(orc_model_params* p);

int orc_camera_look_at(const float origin[3], const float target[3], const float up[3], float width, float height,
                       float fov_rad, float znear, float zfar, float* out);
int orc_camera_from_matrices(const float world_view[16], const float proj[16], float width, float height,
                             float* out);

/* Nearest hit of CastSingleRay for each (x,y) (raytrace3d_bf.cpp:102-174). */
int orc_cast_rays(const orc_mesh* meshes, int n_meshes, const float* cam, const float* xy, int64_t n,
                  uint32_t* prim, uint32_t* inst, uint32_t* geom, float* t, float* u, float* v, float* ray_pos,
                  float* ray_dir);

/* DiffRender::render (drender.h:98-141); images are W*H*3 floats per view. */
int orc_render(const orc_mesh* meshes, int n_meshes, int mode, int spp, const orc_model_params* mp, const float* cams,
               int n_views, float* images);

/* Size/layout of the DMesh gradient block of each differentiable mesh
 * (dmesh.h:35-85): per mesh 9 ints [vertices, instances, pos_off, color_off,
 * tex_off, transform_off, restricted_off, full_size, mesh_id]; a restricted
 * mesh has transform_off -1, every other mesh restricted_off -1. */
int orc_dscene_layout(const orc_mesh* meshes, int n_meshes, int mode, const int32_t* dmesh_ids, int n_ids,
                      int32_t* layout, int64_t* total);

/* DiffRender::d_render (drender.h:144-167).  dscene is accumulated into. */
int orc_d_render(const orc_mesh* meshes, int n_meshes, int mode, int spp, const orc_model_params* mp, const float* cams,
                 int n_views, const float* adjoints, int edge_samples, const int32_t* dmesh_ids, int n_ids,
                 float* dscene);

/* DiffRender::d_render_and_compare (drender.h:169-191). */
int orc_d_render_and_compare(const orc_mesh* meshes, int n_meshes, int mode, int spp, const orc_model_params* mp,
                             const float* cams, int n_views, const float* targets, int edge_samples,
                             const int32_t* dmesh_ids, int n_ids, float* dscene, float* out_images, float* loss);

/* OptimizerParameters (optimizer.h:9-50). */
typedef struct orc_opt_params {
  int32_t alg;
  int32_t decay_period;
  float decay_mult;
  float base_lr, position_lr, textures_lr, transforms_lr;
  int32_t flags;
  int32_t n_dmesh_ids;
  int32_t dmesh_ids[16];
} orc_opt_params;

void orc_opt_params_default(int alg, orc_opt_params* p);

/* OptSimple::Run (optimizer_simple.cpp:272-309).  Meshes are copied; the
 * optimised vertices/colors/textures/transforms of every iteration are
 * written to the optional trajectory arrays (per iteration, per mesh,
 * concatenated; transforms are the matrices the next iteration renders
 * with), the restricted parameters (7 per instance of each restricted mesh)
 * to traj_restricted, and the loss of every iteration to losses. */
int orc_optimize(const orc_mesh* meshes, int n_meshes, int mode, int spp, const orc_model_params* mp, const float* cams,
                 int n_views, const float* targets, const orc_opt_params* p, int iters, float* final_error,
                 float* losses, float* traj_vertices, float* traj_colors, float* traj_textures,
                 float* traj_transforms, float* traj_restricted);

/* TransformR::to_mat (scene.h:99-104): column-major 4x4 of 7 parameters. */
void orc_restricted_to_mat(const float* params7, float* out16);
/* d(to_mat)/d(params), jac[7][12] over the row-major 3x4 part: what the
 * Enzyme forward pass of drender_autodiff.cpp:78-107 computes, derived
 * analytically (the plugin is not available to compile with). */
void orc_restricted_jacobian(const float* params7, float* jac84);

/* Random streams of the edge sampler (qmc.cpp:250-268, drender.h:306-331). */
void orc_prng(int seed, int count, float* out);
void orc_edge_random_table(int num_samples, int num_threads, float* out /* 2*num_samples */);
void orc_hammersley(int n, float* out /* 2n */);

/* Number of OpenMP threads used for the simulated 14-partition loops. */
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
