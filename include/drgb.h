/* drgb: GB300-native differentiable mesh renderer -- C ABI.
 *
 * This is the drop-in boundary for the hot path of the reference renderer
 * (FROL256/diffrender_tutorials): IDiffRender (src/virtual_drender.h:14-26)
 * over Scene/DScene/CamInfo, and the OptSimple optimiser
 * (src/optimizer.h:52-61, src/optimizer_simple.cpp:25-309).  Every entry point
 * takes plain pointers and sizes.  Unless a function says otherwise, data
 * pointers are HOST pointers and the call returns when the results are in
 * host memory; the *_device variants take DEVICE pointers and enqueue work
 * on the renderer's stream without synchronising.
 *
 * All functions return DRGB_OK (0) or a negative error code; the message of
 * the last error on the calling thread is available from drgb_last_error.
 */
#ifndef DRGB_H
#define DRGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DRGB_ABI_VERSION 1

/* Error codes. */
enum {
  DRGB_OK = 0,
  DRGB_ERR_INVALID = -1,      /* bad argument (sizes, ids, null pointers) */
  DRGB_ERR_CUDA = -2,         /* a CUDA call failed */
  DRGB_ERR_OOM = -3,          /* device allocation failed */
  DRGB_ERR_STATE = -4,        /* call out of order (e.g. render before commit) */
  DRGB_ERR_KERNEL = -5,       /* a kernel raised an error flag (traversal stack/limit) */
  DRGB_ERR_UNSUPPORTED = -6,  /* feature not available in this library */
  DRGB_ERR_NO_DEVICE = -7     /* no CUDA device */
};

/* Shading models: the numbering of SHADING_MODEL (src/dmesh.h:16-23) plus two
 * models without a reference counterpart. */
enum {
  DRGB_SILHOUETTE = 1,
  DRGB_VERTEX_COLOR = 2,
  DRGB_TEXTURE_COLOR = 3,
  DRGB_LAMBERT = 4,
  DRGB_PHONG = 5,                 /* shade_lambert.cpp:45-84 */
  DRGB_GGX = 6,                   /* shade_lambert.cpp:86-168 */
  DRGB_PATH_TEST = 7,             /* shade_path_test.cpp:183-289: path tracer, counter-based RNG for rand() */
  DRGB_LAMBERT_POINT_VCOLOR = 16, /* point light, per-vertex albedo, ambient; no reference counterpart */
  DRGB_PATH_DIFFUSE = 17          /* fixed-depth diffuse path tracer with counter RNG; no reference counterpart */
};

/* Optimiser algorithms (OptimizerParameters::OPT_ALGORITHM, src/optimizer.h:11). */
enum { DRGB_GD_NAIVE = 1, DRGB_GD_ADAGRAD = 2, DRGB_GD_RMSPROP = 3, DRGB_GD_ADAM = 4 };
/* Optimiser flags (src/optimizer.h:12-18). */
enum { DRGB_OPT_POS = 1, DRGB_OPT_TFM = 2, DRGB_OPT_COL = 4, DRGB_OPT_TEX = 8 };

/* Renderer options (drgb_renderer_set_option). */
enum {
  DRGB_OPT_TRACE_BRUTEFORCE = 1, /* 1: test every triangle in the reference's loop order instead of the LBVH */
  DRGB_OPT_TILE_W = 2,           /* pixel tile width of the fused forward/adjoint kernel */
  DRGB_OPT_TILE_H = 3,
  DRGB_OPT_USE_GRAPH = 4,        /* 1 (default): optimiser iterations replay a CUDA graph */
  DRGB_OPT_DETERMINISTIC = 5,    /* 1: gradients are summed in a fixed order (records sorted by gradient
                                    index, then segmented sums) instead of by float atomics, so a job's
                                    gradient is bit-identical run to run, alone or in a batch; default 0 */
  DRGB_OPT_ADJOINT_HITS = 6,     /* 1: the interior adjoint reads the primary hits of its samples from a buffer
                                    written by a separate tracing pass (16 bytes per sample) instead of
                                    re-tracing them; 0 (default): re-trace.  Single renderers only. */
  DRGB_OPT_PIXEL_GRID = 7,       /* blocks per SM of the persistent pixel kernel (default 8) */
  DRGB_OPT_EDGE_GRID = 8,        /* blocks per SM of the persistent edge-shading kernel (default 8) */
  DRGB_OPT_BVH_BUILDER = 9,      /* hierarchy topology from the next commit on: 0 LBVH from Morton codes on
                                    the device; binned SAH on the host: 1 (default) two-level when a mesh has
                                    several instances, else one hierarchy; 2 always two-level (one hierarchy
                                    per mesh, shared by its instances, under one over the instances); 3 always
                                    one hierarchy over every triangle.  Boxes are refitted on the device
                                    either way, and a commit of the same triangles keeps the topology */
  DRGB_OPT_BVH_REBUILD = 10,     /* optimiser (and batch, for every job): rebuild the hierarchy topology from
                                    the current vertices every N iterations (default 100; 0: refit only).
                                    The host build overlaps the following iterations; the optimiser uses the
                                    new topology from N/2 iterations after the start on (fixed, not timing
                                    dependent), a batch from the first step after the build completes.
                                    Refitted boxes of moving vertices overlap more and more (icosphere
                                    workload: 55 box tests per ray after 500 steps against 47 with
                                    rebuilds); the hit set does not depend on the topology. */
  DRGB_OPT_TRACE_STEP_LIMIT = 11, /* node visits one ray may make before its traversal gives up (default and
                                    maximum 16,777,216).  A ray that reaches the limit stops with the nearest
                                    hit found so far and the call returns DRGB_ERR_KERNEL ("traversal step
                                    limit"); the renderer stays usable.  The reference has no such bound: its
                                    caster loops over every triangle (raytrace3d_bf.cpp:102-156). */
  DRGB_OPT_EDGE_JACOBIAN = 12,   /* chain rule of the edge term from pixel to vertex positions: 0 (default)
                                    the reference's edge_grad (drender.cpp:31-87): dx/dX and dy/dY only for
                                    the x and y components, through mesh 0's inverse transform; 1 the full
                                    2x3 Jacobian of each endpoint's pixel position, through the transpose of
                                    the edge's own instance transform (exact for any camera and instance) */
  DRGB_OPT_EDGE_SET = 13,        /* edges the boundary term samples: 0 (default) every edge of the
                                    differentiable meshes, in proportion to projected length (the reference,
                                    drender.h:274-285,306-345); 1 per view only silhouette edges (one adjacent
                                    triangle faces the camera, the other faces away) and boundary edges.
                                    Where shading is continuous across edges (interpolated normals and
                                    colours) the other edges contribute only the O(1e-3 px) offset of the
                                    two shading points, so the samples go where the image is discontinuous;
                                    with per-face colours or textures edges inside the silhouette carry real
                                    discontinuities and mode 0 is required */
  DRGB_OPT_PRIMARY_RASTER = 14   /* camera rays and point-light shadow rays: 1 (default) by screen tiles
                                    and light-space cells where that pays -- triangles are binned to the
                                    tiles / cells their projection (with a margin) overlaps, and each ray
                                    runs the reference's ray/triangle test on its tile's or cell's list,
                                    keeping the nearest hit with ties to the lowest triangle, as the
                                    reference's loop does; calls of fewer than about 2 M camera samples
                                    trace, and drgb_optimizer_autotune times both ways; 2 tiles and cells
                                    for every call (no size rule, not switched off by the autotuner); 0
                                    every ray through the hierarchy.  Same hits either way except the reference caster's
                                    clamped-determinant hits, which each method finds only by chance.  Off
                                    for the brute-force caster and stored adjoint hits.  In deterministic
                                    mode the autotuner leaves the choice to the size rule, so a job makes
                                    it alike alone, in a batch and in the server.  Costs 32 bytes per
                                    camera sample of the views (48 for the point-light model) */
};

/* Camera (CamInfo, common_src/camera.h:6-44).  Matrices in LiteMath memory
 * order (column major); mWVP and the inverses used by the caster are derived
 * by the library. */
typedef struct drgb_camera {
  float world_view[16];
  float proj[16];
  float width, height;
} drgb_camera;

/* Fills a camera like CamInfo(origin, target, up, w, h, fov_rad, znear, zfar)
 * (common_src/camera.h:9-22; lookAt/perspectiveMatrix, LiteMath.h:1679-1729). */
int drgb_camera_look_at(const float origin[3], const float target[3], const float up[3], float width, float height,
                        float fov_rad, float znear, float zfar, drgb_camera* out);

/* One mesh and its instances (TriangleMesh + transforms, common_src/scene.h:40-70, 130-138). */
typedef struct drgb_mesh_desc {
  int32_t n_vertices;
  int32_t n_indices;       /* multiple of 3 */
  const float* vertices;   /* 3*n_vertices */
  const float* colors;     /* 3*n_vertices or NULL */
  const float* tc;         /* 2*n_vertices or NULL */
  const float* normals;    /* 3*n_vertices or NULL */
  const float* tangents;   /* 3*n_vertices or NULL */
  const uint32_t* indices; /* n_indices */
  int32_t n_instances;     /* >= 1 */
  const float* transforms; /* 16*n_instances, column major; NULL = one identity instance */
  int32_t tex_w, tex_h, tex_channels; /* first texture; 0 when absent */
  const float* texture;    /* tex_w*tex_h*tex_channels or NULL */
  /* Non-NULL: a RESTRICTED_TRANSFORM mesh (Scene::add_mesh with TransformR,
   * common_src/scene.h:91-116,140-148), 7 floats per instance
   * {translate x,y,z; rotate x,y,z (radians); scale}.  The instance matrices
   * are TransformR::to_mat of these (`transforms` is ignored) and the
   * gradient holds 7 values per instance in place of the 12 matrix entries. */
  const float* restricted;
} drgb_mesh_desc;

typedef struct drgb_scene_desc {
  int32_t n_meshes;
  const drgb_mesh_desc* meshes;
} drgb_scene_desc;

/* Constants of the two models without a reference counterpart; of these,
 * PATH_TEST (whose constants are the reference's) uses only `seed`, the
 * key of its counter-based random numbers. */
typedef struct drgb_model_params {
  float light_pos[3];
  float light_intensity;
  float ambient;
  int32_t path_depth;
  uint32_t seed;
} drgb_model_params;

/* OptimizerParameters (src/optimizer.h:9-50). */
typedef struct drgb_opt_params {
  int32_t alg;
  int32_t decay_period;
  float decay_mult;
  float base_lr, position_lr, textures_lr, transforms_lr;
  int32_t flags;
  int32_t n_dmesh_ids;
  int32_t dmesh_ids[16];
} drgb_opt_params;

typedef struct drgb_renderer drgb_renderer;

/* ---- library ------------------------------------------------------------ */
int drgb_abi_version(void);
/* Message of the last failed call on this thread (always NUL-terminated). */
int drgb_last_error(char* buf, size_t len);
/* Number of kernels this library launched since load (all threads). */
int64_t drgb_kernel_launches(void);
/* Test hook, no counterpart in the reference: the device exclusive scan of
 * n 32-bit counters that the radix sorts of the hierarchy build, the
 * edge-sample queue and the deterministic reduction use (host arrays in and
 * out, current device, synchronous). */
int drgb_debug_exclusive_scan(const uint32_t* counts, int n, uint32_t* out);

/* ---- renderer: IDiffRender (src/virtual_drender.h:14-26) ----------------- */

/* MakeDifferentialRenderer(DiffRenderSettings{mode, spp}) + init
 * (src/drender.cpp:89-147, src/drender.h:79-88). */
int drgb_renderer_create(int shading_model, int spp, int device, drgb_renderer** out);
int drgb_renderer_destroy(drgb_renderer* r);
int drgb_renderer_set_option(drgb_renderer* r, int option, int64_t value);
int drgb_renderer_set_model_params(drgb_renderer* r, const drgb_model_params* p);
/* CUDA stream (cudaStream_t) the renderer enqueues on. */
void* drgb_renderer_stream(drgb_renderer* r);

/* IDiffRender::commit (src/drender.h:91-96): uploads the scene, flattens it
 * and builds the ray-tracing hierarchy (a scene with the same triangles keeps
 * its topology and refits it; the device buffers of same-sized meshes are
 * reused).  Returns once the scene's arrays have been read: at once for
 * pageable host memory, with the flattening and refit left running on the
 * renderer stream ahead of the next call; after that stream has finished
 * when an array is page-locked. */
int drgb_commit(drgb_renderer* r, const drgb_scene_desc* scene);

/* IDiffRender::render (src/drender.h:98-141): images are width*height*3
 * floats per view, concatenated in view order. */
int drgb_render(drgb_renderer* r, const drgb_camera* cams, int n_views, float* images);

/* Layout of the gradient vector of DScene(scene, mode, dmesh_ids)
 * (src/dmesh.h:35-85, 155-222): 9 ints per differentiable mesh
 * [vertices, instances, pos_off, color_off, tex_off, transform_off,
 *  restricted_off, full_size, mesh_id]; *total = sum of full sizes.  A
 * restricted mesh has transform_off -1, any other mesh restricted_off -1. */
int drgb_dscene_layout(drgb_renderer* r, const int32_t* dmesh_ids, int n_ids, int32_t* layout, int64_t* total);

/* IDiffRender::d_render (src/drender.h:144-167): accumulates (+=) into the
 * gradient vector dscene (layout of drgb_dscene_layout). */
int drgb_d_render(drgb_renderer* r, const drgb_camera* cams, const float* adjoints, int n_views,
                  int edge_samples_in_total, const int32_t* dmesh_ids, int n_ids, float* dscene);

/* IDiffRender::d_render_and_compare (src/drender.h:169-191): renders, forms
 * the MSE loss and its adjoint 2*(I-T), clears dscene and fills it with the
 * interior + edge gradient; out_images may be NULL. */
int drgb_d_render_and_compare(drgb_renderer* r, const drgb_camera* cams, const float* targets, int n_views,
                              int edge_samples_in_total, const int32_t* dmesh_ids, int n_ids, float* dscene,
                              float* out_images, float* loss);

/* Same with device pointers (targets, dscene, out_images, loss may be device
 * memory the caller owns): no copies through host memory.  The work is
 * enqueued on the renderer stream and the call returns when that stream has
 * finished it; kernel error flags are left for the next host-pointer call
 * to report. */
int drgb_d_render_and_compare_device(drgb_renderer* r, const drgb_camera* cams, const float* d_targets, int n_views,
                                     int edge_samples_in_total, const int32_t* dmesh_ids, int n_ids, float* d_dscene,
                                     float* d_out_images, float* d_loss);

/* No counterpart in the reference.  The same computation and outputs as
 * drgb_d_render_and_compare_device (gradient vector and loss written to
 * caller-owned device memory), for callers that cannot allocate GPU memory
 * while they run: programs that take all device memory from a pool or
 * budget of their own and forbid cudaMalloc after start-up, and loops that
 * must not pay for an allocation (or the synchronisation it can cause)
 * mid-run.  The call makes no cudaMalloc/cudaFree; its per-call buffers come
 * from one 32 MiB array compiled into the library.  The first call on a
 * device looks the array's address up (the runtime may load the array onto
 * the device then; it stays until exit); make that first call before any
 * stream capture.  Calls needing more than the array (roughly: beyond one
 * 512x512 view with 262,144 edge samples) return DRGB_ERR_INVALID.  All
 * calls share the array, so calls that overlap on the GPU race.  Each call
 * rebuilds the edge list and the replayed random numbers on the host, copies
 * them from pageable memory and waits for the renderer's stream before it
 * returns.  The scene must have been committed (drgb_commit) beforehand. */
int drgb_d_render_and_compare_noalloc(drgb_renderer* r, const drgb_camera* cams, const float* d_targets,
                                      int n_views, int edge_samples_in_total, const int32_t* dmesh_ids, int n_ids,
                                      float* d_dscene, float* d_loss);

/* Per-sample nearest hits of camera rays through (x,y) pixel positions
 * (IRayTracer::CastSingleRay, raytrace_src/raytrace.h:31-41): prim, inst,
 * geom, t, u, v arrays of n entries (host). */
int drgb_cast_rays(drgb_renderer* r, const drgb_camera* cam, const float* xy, int64_t n, uint32_t* prim,
                   uint32_t* inst, uint32_t* geom, float* t, float* u, float* v);

/* ---- optimiser: IOptimizer / OptSimple (src/optimizer.h:52-61) ---------- */
int drgb_opt_params_default(int alg, drgb_opt_params* out);
/* IOptimizer::Init: scene, views and target images (host). */
int drgb_optimizer_init(drgb_renderer* r, const drgb_scene_desc* scene, const drgb_camera* cams, const float* targets,
                        int n_views, const drgb_opt_params* p);
/* IOptimizer::Run: iterations of d_render_and_compare + OptStep +
 * OptUpdateScene + StepDecay, all on the device; final_error = loss of the
 * last iteration (optimizer_simple.cpp:272-309).  losses (n_iters floats,
 * may be NULL) receives every iteration's loss. */
int drgb_optimizer_run(drgb_renderer* r, int64_t n_iters, float* final_error, float* losses);
/* Enqueue n_iters iterations without synchronising (device-resident loop). */
int drgb_optimizer_run_async(drgb_renderer* r, int64_t n_iters);
/* Current optimised parameters of one mesh (host arrays, may be NULL). */
int drgb_optimizer_get_mesh(drgb_renderer* r, int mesh_id, float* vertices, float* colors, float* texture,
                            float* transforms);
/* Current TransformR parameters of a restricted mesh (7 per instance,
 * Scene::get_restricted_transform, scene.h:191); DRGB_ERR_INVALID for any
 * other mesh. */
int drgb_optimizer_get_restricted(drgb_renderer* r, int mesh_id, float* params);

/* ---- batched optimisation (no reference counterpart: the reference runs one
 * OptSimple at a time, src/tests.cpp:125-204).  A batch advances many
 * independent optimisation jobs -- each one the equivalent of
 * IOptimizer::Init + Run (src/optimizer.h:52-61) -- with one fused launch
 * sequence per iteration, replayed from a CUDA graph.  Every job is set up
 * exactly as drgb_optimizer_init sets up a plain optimiser, so a job computes
 * the same alone and in a batch (up to the order of floating-point atomic
 * additions). ------------------------------------------------------------- */
typedef struct drgb_batch drgb_batch;
int drgb_batch_create(int device, drgb_batch** out);
int drgb_batch_destroy(drgb_batch* b);
void* drgb_batch_stream(drgb_batch* b);
/* Adds a job (scene, views, host target images, optimiser parameters;
 * model_params may be NULL).  Returns its id in *job_id. */
int drgb_batch_add_job(drgb_batch* b, int shading_model, int spp, const drgb_model_params* model_params,
                       const drgb_scene_desc* scene, const drgb_camera* cams, const float* targets, int n_views,
                       const drgb_opt_params* p, int32_t* job_id);
int drgb_batch_remove_job(drgb_batch* b, int32_t job_id);
int drgb_batch_size(drgb_batch* b);
/* DRGB_OPT_USE_GRAPH, or DRGB_OPT_DETERMINISTIC / DRGB_OPT_BVH_REBUILD / DRGB_OPT_PRIMARY_RASTER for
 * every job, present and future */
int drgb_batch_set_option(drgb_batch* b, int option, int64_t value);
/* n_iters iterations of every job: enqueue only / enqueue and wait. */
int drgb_batch_run_async(drgb_batch* b, int64_t n_iters);
int drgb_batch_run(drgb_batch* b, int64_t n_iters);
int drgb_batch_sync(drgb_batch* b);
/* Losses of iterations [first, first+n) of a job; *iters_done = iterations run. */
int drgb_batch_job_losses(drgb_batch* b, int32_t job_id, int64_t first, int64_t n, float* out, int64_t* iters_done);
int drgb_batch_get_mesh(drgb_batch* b, int32_t job_id, int mesh_id, float* vertices, float* colors, float* texture,
                        float* transforms);
int drgb_batch_get_restricted(drgb_batch* b, int32_t job_id, int mesh_id, float* params);
/* Device memory held by a job (for admission against a memory budget). */
int64_t drgb_batch_job_device_bytes(drgb_batch* b, int32_t job_id);

/* ---- serving (no reference counterpart; each job is one IOptimizer::Init +
 * Run(n_steps), src/optimizer.h:52-61).  Jobs are submitted at any time and
 * queue in arrival order; a job is admitted when a slot is free and its
 * device memory fits the budget; every admitted job advances one iteration
 * per batched step (continuous batching: jobs join and leave between steps,
 * and new jobs are set up on their own streams while a step runs).  A
 * finished job's final meshes and loss history are copied to host memory and
 * its device memory is freed.  With start_worker = 1 a worker thread steps
 * the batch whenever jobs are queued or resident; otherwise the caller calls
 * drgb_server_step. ------------------------------------------------------- */
typedef struct drgb_server drgb_server;

typedef struct drgb_server_config {
  int32_t device;
  int32_t max_jobs;         /* resident jobs at most; <= 0: no limit */
  int64_t hbm_budget_bytes; /* device memory of resident jobs at most */
  int32_t start_worker;     /* 1: step from a worker thread */
  int32_t deterministic;    /* 1: jobs use DRGB_OPT_DETERMINISTIC */
} drgb_server_config;

enum { DRGB_JOB_QUEUED = 0, DRGB_JOB_RUNNING = 1, DRGB_JOB_DONE = 2, DRGB_JOB_FAILED = 3 };

typedef struct drgb_job_info {
  int32_t state;        /* DRGB_JOB_* */
  int32_t error;        /* error code of a failed job */
  int64_t steps, steps_done;
  double t_submit, t_admit, t_done; /* seconds on the server's clock; -1 until reached */
  int64_t device_bytes; /* measured once admitted, estimated before */
  float final_loss;
} drgb_job_info;

typedef struct drgb_server_stats {
  int32_t queued, running, done, failed;
  int64_t bytes_in_use, bytes_budget, bytes_peak;
  int64_t batch_steps;    /* batched iterations run */
  int64_t job_iterations; /* iterations summed over jobs */
  double busy_seconds;    /* device time of the batched iterations (CUDA events) */
  double now;             /* the server's clock */
} drgb_server_stats;

int drgb_server_create(const drgb_server_config* cfg, drgb_server** out);
/* Stops the worker and frees every job. */
int drgb_server_destroy(drgb_server* s);
/* Queues a job; inputs are copied, so the caller may free them on return.
 * DRGB_ERR_OOM when the job alone exceeds the budget. */
int drgb_server_submit(drgb_server* s, int shading_model, int spp, const drgb_model_params* model_params,
                       const drgb_scene_desc* scene, const drgb_camera* cams, const float* targets, int n_views,
                       const drgb_opt_params* p, int64_t n_steps, int32_t* ticket);
/* Without a worker: admit, run one batched iteration, retire finished jobs.
 * *n_running (may be NULL) = jobs resident after the step. */
int drgb_server_step(drgb_server* s, int32_t* n_running);
/* Blocks until the job (ticket > 0) or every submitted job (ticket = 0) is
 * done or failed; DRGB_ERR_STATE after timeout_s seconds (< 0: no limit). */
int drgb_server_wait(drgb_server* s, int32_t ticket, double timeout_s);
int drgb_server_job_info(drgb_server* s, int32_t ticket, drgb_job_info* out);
int drgb_server_job_losses(drgb_server* s, int32_t ticket, int64_t first, int64_t n, float* out);
int drgb_server_get_mesh(drgb_server* s, int32_t ticket, int mesh_id, float* vertices, float* colors,
                         float* texture, float* transforms);
int drgb_server_get_restricted(drgb_server* s, int32_t ticket, int mesh_id, float* params);
/* Forgets a finished job's results. */
int drgb_server_release(drgb_server* s, int32_t ticket);
int drgb_server_get_stats(drgb_server* s, drgb_server_stats* out);
/* Device time (ms) and resident job count of batched steps [first, first+n). */
int drgb_server_step_times(drgb_server* s, int64_t first, int64_t n, float* ms, int32_t* jobs);
/* Device bytes a job of this shape needs (an upper estimate used for admission). */
int64_t drgb_estimate_job_bytes(int shading_model, int spp, const drgb_scene_desc* scene, const drgb_camera* cams,
                                int n_views);

/* ---- measurement (no reference counterpart: the reference prints wall-clock
 * ms/iter only, src/main.cpp:218-224, src/tests.cpp:136-203) -------------- */
/* Runs n_iters optimiser iterations phase by phase (no graph) and returns the
 * mean CUDA-event time of each phase on the renderer stream, in ms:
 * out_ms[0] forward+loss+interior adjoint, [1] edge sampling, [2] optimiser
 * step, [3] flatten+LBVH refit, [4] whole iteration. */
int drgb_optimizer_profile(drgb_renderer* r, int n_iters, float* out_ms);
/* Work of one optimiser iteration's pixel and edge passes, counted by an
 * instrumented replay: counts[0] rays (traced, or resolved against a screen
 * tile or light cell), [1] ray/box tests, [2] ray/triangle tests, [3] edge
 * samples shaded, [4] footprint tests of the tile and cell lists (5 entries). */
int drgb_count_work(drgb_renderer* r, uint64_t* counts);

/* ---- autotuning (no reference counterpart) ------------------------------
 * Times the gradient passes of the optimiser's views (no update: the
 * optimiser's state does not change) for candidate work-item shapes (32 or
 * 64 samples per item) and persistent grid sizes (2, 4, 8, 16 blocks per SM
 * for the pixel and the edge-shading kernels), by coordinate descent, and
 * keeps the fastest; with DRGB_OPT_PRIMARY_RASTER = 1 it first times the
 * camera and shadow rays by tiles and cells against traversal.  chosen (may
 * be NULL) receives 5 values: tile_w, tile_h, pixel blocks per SM, edge
 * blocks per SM, 1 if tiles and cells are used; best_ms the mean time of the
 * passes. */
int drgb_optimizer_autotune(drgb_renderer* r, int trial_iters, int32_t* chosen, float* best_ms);
/* The same for a batch: the grid sizes of its shared launches (2 ints). */
int drgb_batch_autotune(drgb_batch* b, int trial_iters, int32_t* chosen, float* best_ms);

#ifdef __cplusplus
}
#endif
#endif /* DRGB_H */
