/* CPU oracle for the differentiable mesh renderer hot path -- TEST
 * INFRASTRUCTURE ONLY (checker and timed CPU baseline; never shipped).
 *
 * A plain-C restatement of the reference renderer (FROL256/diffrender_tutorials)
 * built with its brute-force caster.  Every function cites the reference
 * file:line it follows.  Floating-point expressions keep the reference's
 * operation order; build with -ffp-contract=off so that no multiply-add is
 * fused (x86-64 g++ without -march emits none, which is what the reference
 * numbers were produced with).
 *
 * Accumulation of gradients replays the reference's OpenMP layout: the pixel
 * loop and the edge-sample loop are split into 14 contiguous static blocks
 * (MAXTHREADS, src/drender.h:10-13; libgomp static schedule), each block sums
 * into its own buffer in iteration order, and the buffers are added in block
 * order.  Real threads (OpenMP, when available) execute whole blocks, so the
 * result does not depend on how many host threads run it.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define REF_THREADS 14 /* MAXTHREADS, src/drender.h:12 */
#define ORC_CHUNK 16   /* triangles per vectorised step of the brute-force caster */

typedef struct { float x, y, z; } f3;
typedef struct { float x, y; } f2;

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }

/* ---------------------------------------------------------------------------
 * LiteMath restatement (common_src/LiteMath.h).  Scalar IEEE operations in
 * the order written there.
 * ------------------------------------------------------------------------- */
static inline f3 v3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 add3(f3 a, f3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 sub3(f3 a, f3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 mul3(f3 a, f3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline f3 scl3(f3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline f3 div3s(f3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
/* LiteMath.h:792 */
static inline float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* LiteMath.h:794-795 */
static inline float len3(f3 a) { return sqrtf(dot3(a, a)); }
static inline f3 norm3(f3 a) { float inv = 1.0f / len3(a); return scl3(a, inv); }
/* LiteMath.h:816-821: shuffle_yzx(a*b_yzx - a_yzx*b) */
static inline f3 cross3(f3 a, f3 b) {
  float dx = a.x * b.y - a.y * b.x;
  float dy = a.y * b.z - a.z * b.y;
  float dz = a.z * b.x - a.x * b.z;
  return v3(dy, dz, dx);
}
/* LiteMath.h:109-114 */
static inline float signf_ref(float x) {
  if (x == 0.0f) return 0.0f;
  else if (x < 0.0f) return -1.0f;
  else return 1.0f;
}
static inline float maxf_ref(float a, float b) { return (a < b) ? b : a; } /* std::max */
static inline float minf_ref(float a, float b) { return (b < a) ? b : a; } /* std::min */
/* LiteMath.h:84 */
static inline float clampf_ref(float u, float a, float b) { return minf_ref(maxf_ref(a, u), b); }
static inline int clampi(int u, int a, int b) { int m = (a < u) ? u : a; return (b < m) ? b : m; }
static inline f2 v2(float x, float y) { f2 r = {x, y}; return r; }
static inline f2 add2(f2 a, f2 b) { return v2(a.x + b.x, a.y + b.y); }
static inline f2 sub2(f2 a, f2 b) { return v2(a.x - b.x, a.y - b.y); }
static inline f2 scl2(f2 a, float s) { return v2(a.x * s, a.y * s); }
static inline float dot2(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
static inline float len2(f2 a) { return sqrtf(dot2(a, a)); }

/* Column-major 4x4: element (row r, col c) at m[4c + r] (LiteMath.h:1367-1433). */
#define M(m, r, c) ((m)[4 * (c) + (r)])

/* mat4_colmajor_mul_vec4, LiteMath.h:1342-1348 */
static inline void mat_vec4(const float* B, const float* V, float* R) {
  for (int i = 0; i < 4; i++) R[i] = V[0] * B[i] + V[1] * B[4 + i] + V[2] * B[8 + i] + V[3] * B[12 + i];
}
/* float4x4 * float3 (w = 1), LiteMath.h:1451-1457 */
static inline f3 mat_pt(const float* m, f3 p) {
  float V[4] = {p.x, p.y, p.z, 1.0f}, R[4];
  mat_vec4(m, V, R);
  return v3(R[0], R[1], R[2]);
}
/* float4x4 * float4x4, LiteMath.h:1536-1549 */
static void mat_mul(const float* a, const float* b, float* out) {
  float tmp[16];
  for (int c = 0; c < 4; c++) mat_vec4(a, b + 4 * c, tmp + 4 * c);
  memcpy(out, tmp, sizeof(tmp));
}
/* Cofactor inverse, LiteMath.h:1551-1633 (same pairing and accumulation order). */
static void mat_inverse(const float* m1, float* out) {
  float tmp[12], m[16];
  tmp[0] = M(m1, 2, 2) * M(m1, 3, 3);
  tmp[1] = M(m1, 2, 3) * M(m1, 3, 2);
  tmp[2] = M(m1, 2, 1) * M(m1, 3, 3);
  tmp[3] = M(m1, 2, 3) * M(m1, 3, 1);
  tmp[4] = M(m1, 2, 1) * M(m1, 3, 2);
  tmp[5] = M(m1, 2, 2) * M(m1, 3, 1);
  tmp[6] = M(m1, 2, 0) * M(m1, 3, 3);
  tmp[7] = M(m1, 2, 3) * M(m1, 3, 0);
  tmp[8] = M(m1, 2, 0) * M(m1, 3, 2);
  tmp[9] = M(m1, 2, 2) * M(m1, 3, 0);
  tmp[10] = M(m1, 2, 0) * M(m1, 3, 1);
  tmp[11] = M(m1, 2, 1) * M(m1, 3, 0);
  M(m, 0, 0) = tmp[0] * M(m1, 1, 1) + tmp[3] * M(m1, 1, 2) + tmp[4] * M(m1, 1, 3);
  M(m, 0, 0) -= tmp[1] * M(m1, 1, 1) + tmp[2] * M(m1, 1, 2) + tmp[5] * M(m1, 1, 3);
  M(m, 1, 0) = tmp[1] * M(m1, 1, 0) + tmp[6] * M(m1, 1, 2) + tmp[9] * M(m1, 1, 3);
  M(m, 1, 0) -= tmp[0] * M(m1, 1, 0) + tmp[7] * M(m1, 1, 2) + tmp[8] * M(m1, 1, 3);
  M(m, 2, 0) = tmp[2] * M(m1, 1, 0) + tmp[7] * M(m1, 1, 1) + tmp[10] * M(m1, 1, 3);
  M(m, 2, 0) -= tmp[3] * M(m1, 1, 0) + tmp[6] * M(m1, 1, 1) + tmp[11] * M(m1, 1, 3);
  M(m, 3, 0) = tmp[5] * M(m1, 1, 0) + tmp[8] * M(m1, 1, 1) + tmp[11] * M(m1, 1, 2);
  M(m, 3, 0) -= tmp[4] * M(m1, 1, 0) + tmp[9] * M(m1, 1, 1) + tmp[10] * M(m1, 1, 2);
  M(m, 0, 1) = tmp[1] * M(m1, 0, 1) + tmp[2] * M(m1, 0, 2) + tmp[5] * M(m1, 0, 3);
  M(m, 0, 1) -= tmp[0] * M(m1, 0, 1) + tmp[3] * M(m1, 0, 2) + tmp[4] * M(m1, 0, 3);
  M(m, 1, 1) = tmp[0] * M(m1, 0, 0) + tmp[7] * M(m1, 0, 2) + tmp[8] * M(m1, 0, 3);
  M(m, 1, 1) -= tmp[1] * M(m1, 0, 0) + tmp[6] * M(m1, 0, 2) + tmp[9] * M(m1, 0, 3);
  M(m, 2, 1) = tmp[3] * M(m1, 0, 0) + tmp[6] * M(m1, 0, 1) + tmp[11] * M(m1, 0, 3);
  M(m, 2, 1) -= tmp[2] * M(m1, 0, 0) + tmp[7] * M(m1, 0, 1) + tmp[10] * M(m1, 0, 3);
  M(m, 3, 1) = tmp[4] * M(m1, 0, 0) + tmp[9] * M(m1, 0, 1) + tmp[10] * M(m1, 0, 2);
  M(m, 3, 1) -= tmp[5] * M(m1, 0, 0) + tmp[8] * M(m1, 0, 1) + tmp[11] * M(m1, 0, 2);
  tmp[0] = M(m1, 0, 2) * M(m1, 1, 3);
  tmp[1] = M(m1, 0, 3) * M(m1, 1, 2);
  tmp[2] = M(m1, 0, 1) * M(m1, 1, 3);
  tmp[3] = M(m1, 0, 3) * M(m1, 1, 1);
  tmp[4] = M(m1, 0, 1) * M(m1, 1, 2);
  tmp[5] = M(m1, 0, 2) * M(m1, 1, 1);
  tmp[6] = M(m1, 0, 0) * M(m1, 1, 3);
  tmp[7] = M(m1, 0, 3) * M(m1, 1, 0);
  tmp[8] = M(m1, 0, 0) * M(m1, 1, 2);
  tmp[9] = M(m1, 0, 2) * M(m1, 1, 0);
  tmp[10] = M(m1, 0, 0) * M(m1, 1, 1);
  tmp[11] = M(m1, 0, 1) * M(m1, 1, 0);
  M(m, 0, 2) = tmp[0] * M(m1, 3, 1) + tmp[3] * M(m1, 3, 2) + tmp[4] * M(m1, 3, 3);
  M(m, 0, 2) -= tmp[1] * M(m1, 3, 1) + tmp[2] * M(m1, 3, 2) + tmp[5] * M(m1, 3, 3);
  M(m, 1, 2) = tmp[1] * M(m1, 3, 0) + tmp[6] * M(m1, 3, 2) + tmp[9] * M(m1, 3, 3);
  M(m, 1, 2) -= tmp[0] * M(m1, 3, 0) + tmp[7] * M(m1, 3, 2) + tmp[8] * M(m1, 3, 3);
  M(m, 2, 2) = tmp[2] * M(m1, 3, 0) + tmp[7] * M(m1, 3, 1) + tmp[10] * M(m1, 3, 3);
  M(m, 2, 2) -= tmp[3] * M(m1, 3, 0) + tmp[6] * M(m1, 3, 1) + tmp[11] * M(m1, 3, 3);
  M(m, 3, 2) = tmp[5] * M(m1, 3, 0) + tmp[8] * M(m1, 3, 1) + tmp[11] * M(m1, 3, 2);
  M(m, 3, 2) -= tmp[4] * M(m1, 3, 0) + tmp[9] * M(m1, 3, 1) + tmp[10] * M(m1, 3, 2);
  M(m, 0, 3) = tmp[2] * M(m1, 2, 2) + tmp[5] * M(m1, 2, 3) + tmp[1] * M(m1, 2, 1);
  M(m, 0, 3) -= tmp[4] * M(m1, 2, 3) + tmp[0] * M(m1, 2, 1) + tmp[3] * M(m1, 2, 2);
  M(m, 1, 3) = tmp[8] * M(m1, 2, 3) + tmp[0] * M(m1, 2, 0) + tmp[7] * M(m1, 2, 2);
  M(m, 1, 3) -= tmp[6] * M(m1, 2, 2) + tmp[9] * M(m1, 2, 3) + tmp[1] * M(m1, 2, 0);
  M(m, 2, 3) = tmp[6] * M(m1, 2, 1) + tmp[11] * M(m1, 2, 3) + tmp[3] * M(m1, 2, 0);
  M(m, 2, 3) -= tmp[10] * M(m1, 2, 3) + tmp[2] * M(m1, 2, 0) + tmp[7] * M(m1, 2, 1);
  M(m, 3, 3) = tmp[10] * M(m1, 2, 2) + tmp[4] * M(m1, 2, 0) + tmp[9] * M(m1, 2, 1);
  M(m, 3, 3) -= tmp[8] * M(m1, 2, 1) + tmp[11] * M(m1, 2, 2) + tmp[5] * M(m1, 2, 0);
  const float k = 1.0f / (M(m1, 0, 0) * M(m, 0, 0) + M(m1, 0, 1) * M(m, 1, 0) + M(m1, 0, 2) * M(m, 2, 0) +
                          M(m1, 0, 3) * M(m, 3, 0));
  for (int i = 0; i < 16; i++) out[i] = m[i] * k;
}

static void mat_identity(float* m) {
  memset(m, 0, 16 * sizeof(float));
  m[0] = m[5] = m[10] = m[15] = 1.0f;
}

/* ---------------------------------------------------------------------------
 * Restricted transforms (TransformR, scene.h:91-116).
 * ------------------------------------------------------------------------- */
/* to_mat: translate4x4(t) * rotate4x4Z(rz) * rotate4x4Y(ry) * rotate4x4X(rx)
 * * scale4x4(s), products left to right (LiteMath.h:1474-1549). */
void orc_restricted_to_mat(const float* p, float* out) {
  float T[16], Rz[16], Ry[16], Rx[16], S[16], a[16], b[16];
  mat_identity(T);
  M(T, 0, 3) = p[0]; M(T, 1, 3) = p[1]; M(T, 2, 3) = p[2];
  mat_identity(Rz);
  M(Rz, 0, 0) = cosf(p[5]); M(Rz, 1, 0) = sinf(p[5]); M(Rz, 0, 1) = -sinf(p[5]); M(Rz, 1, 1) = cosf(p[5]);
  mat_identity(Ry);
  M(Ry, 0, 0) = cosf(p[4]); M(Ry, 2, 0) = -sinf(p[4]); M(Ry, 0, 2) = sinf(p[4]); M(Ry, 2, 2) = cosf(p[4]);
  mat_identity(Rx);
  M(Rx, 1, 1) = cosf(p[3]); M(Rx, 2, 1) = sinf(p[3]); M(Rx, 1, 2) = -sinf(p[3]); M(Rx, 2, 2) = cosf(p[3]);
  mat_identity(S);
  M(S, 0, 0) = p[6]; M(S, 1, 1) = p[6]; M(S, 2, 2) = p[6];
  mat_mul(T, Rz, a);
  mat_mul(a, Ry, b);
  mat_mul(b, Rx, a);
  mat_mul(a, S, out);
}

/* Row-major 3x4 product with translation, `mul` of drender_autodiff.cpp:22-43. */
static void mul34(const float* a, const float* b, float* out) {
  float r[12];
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) r[4 * i + j] = a[4 * i + 0] * b[j] + a[4 * i + 1] * b[4 + j] + a[4 * i + 2] * b[8 + j];
    r[4 * i + 3] = a[4 * i + 0] * b[3] + a[4 * i + 1] * b[7] + a[4 * i + 2] * b[11] + a[4 * i + 3];
  }
  memcpy(out, r, sizeof(r));
}

/* dmat_dtransforms_jac_f (drender_autodiff.cpp:78-95) builds
 * out = Rz (Ry (Rx S)) + translation; its derivative for each parameter is
 * the same chain with one factor replaced by that factor's derivative
 * (d/dr of {cos r, sin r} = {-sin r, cos r}), the translation entries have
 * derivative 1.  Row k of jac is d out / d params[k]. */
void orc_restricted_jacobian(const float* x, float* jac) {
  const float sx = sinf(x[3]), cx = cosf(x[3]), sy = sinf(x[4]), cy = cosf(x[4]), sz = sinf(x[5]), cz = cosf(x[5]);
  const float S[12] = {x[6], 0, 0, 0, 0, x[6], 0, 0, 0, 0, x[6], 0};
  const float dS[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  const float Rx[12] = {1, 0, 0, 0, 0, cx, -sx, 0, 0, sx, cx, 0};
  const float Ry[12] = {cy, 0, sy, 0, 0, 1, 0, 0, -sy, 0, cy, 0};
  const float Rz[12] = {cz, -sz, 0, 0, sz, cz, 0, 0, 0, 0, 1, 0};
  const float dRx[12] = {0, 0, 0, 0, 0, -sx, -cx, 0, 0, cx, -sx, 0};
  const float dRy[12] = {-sy, 0, cy, 0, 0, 0, 0, 0, -cy, 0, -sy, 0};
  const float dRz[12] = {-sz, -cz, 0, 0, cz, -sz, 0, 0, 0, 0, 0, 0};
  float a[12], b[12];
  memset(jac, 0, 84 * sizeof(float));
  jac[0 * 12 + 3] = 1.0f;
  jac[1 * 12 + 7] = 1.0f;
  jac[2 * 12 + 11] = 1.0f;
  mul34(dRx, S, a); mul34(Ry, a, b); mul34(Rz, b, jac + 3 * 12);
  mul34(Rx, S, a); mul34(dRy, a, b); mul34(Rz, b, jac + 4 * 12);
  mul34(Rx, S, a); mul34(Ry, a, b); mul34(dRz, b, jac + 5 * 12);
  mul34(Rx, dS, a); mul34(Ry, a, b); mul34(Rz, b, jac + 6 * 12);
}

/* ---------------------------------------------------------------------------
 * Camera: CamInfo (common_src/camera.h:9-44), lookAt / perspectiveMatrix
 * (LiteMath.h:1679-1729), BruteForce3D::SetCamera (raytrace3d_bf.cpp:93-100).
 * ------------------------------------------------------------------------- */
static void look_at(f3 eye, f3 center, f3 up, float* Mo) {
  f3 z = v3(eye.x - center.x, eye.y - center.y, eye.z - center.z);
  z = norm3(z);
  f3 y = up;
  f3 x = cross3(y, z);
  y = cross3(z, x);
  x = norm3(x);
  y = norm3(y);
  float m[16] = {x.x, y.x, z.x, 0.0f, x.y, y.y, z.y, 0.0f, x.z, y.z, z.z, 0.0f,
                 -x.x * eye.x - x.y * eye.y - x.z * eye.z, -y.x * eye.x - y.y * eye.y - y.z * eye.z,
                 -z.x * eye.x - z.y * eye.y - z.z * eye.z, 1.0f};
  memcpy(Mo, m, sizeof(m));
}

/* tanf through double: correctly rounded for the arguments used here and
 * identical on every host libm; tests pin it against the reference build. */
static float tanf_cr(float x) { return (float)tan((double)x); }

static void perspective(float fovy, float aspect, float zNear, float zFar, float* Mo) {
  const float ymax = zNear * tanf_cr(fovy * 3.14159265358979323846f / 360.0f);
  const float xmax = ymax * aspect;
  const float left = -xmax, right = +xmax, bottom = -ymax, top = +ymax;
  const float temp = 2.0f * zNear, temp2 = right - left, temp3 = top - bottom, temp4 = zFar - zNear;
  float m[16] = {temp / temp2, 0.0f, 0.0f, 0.0f,
                 0.0f, temp / temp3, 0.0f, 0.0f,
                 (right + left) / temp2, (top + bottom) / temp3, (-zFar - zNear) / temp4, -1.0f,
                 0.0f, 0.0f, (-temp * zFar) / temp4, 0.0f};
  memcpy(Mo, m, sizeof(m));
}

int orc_camera_from_matrices(const float wv[16], const float proj[16], float width, float height, float* out) {
  memcpy(out, wv, 16 * sizeof(float));
  memcpy(out + 16, proj, 16 * sizeof(float));
  mat_mul(proj, wv, out + 32); /* CamInfo::commit: mProj*mWorldView */
  mat_inverse(proj, out + 48);
  mat_inverse(wv, out + 64);
  out[80] = width;
  out[81] = height;
  return 0;
}

int orc_camera_look_at(const float o[3], const float t[3], const float u[3], float width, float height, float fov_rad,
                       float znear, float zfar, float* out) {
  const float DEG_TO_RAD = 3.14159265358979323846f / 180.0f; /* LiteMath.h:48 */
  float wv[16], pr[16];
  perspective(fov_rad / DEG_TO_RAD, width / height, znear, zfar, pr);
  look_at(v3(o[0], o[1], o[2]), v3(t[0], t[1], t[2]), v3(u[0], u[1], u[2]), wv);
  return orc_camera_from_matrices(wv, pr, width, height, out);
}

/* ---------------------------------------------------------------------------
 * Prepared scene (Scene::prepare_for_render, scene_utils.cpp:98-173).
 * ------------------------------------------------------------------------- */
typedef struct {
  const orc_mesh* meshes;
  int n_meshes;
  int n_blocks;      /* (mesh, instance) pairs */
  int* mesh_block0;  /* first block of each mesh */
  int* block_off;    /* flattened vertex offset of each block */
  int* block_mesh;
  int total;
  f3 *pos, *orig, *col, *nrm, *tng;
  f2* tc;
  float* tr;     /* 16 per block */
  float* tr_inv; /* 16 per block */
  /* traced triangles: transform applied to prepared positions again, as the
   * brute-force caster does (raytrace3d_bf.cpp:116-125) */
  int n_tris;
  int* tri_block;
  int* tri_prim;
  f3 *ta, *te1, *te2;
  int* tri_gid; /* 3 global vertex ids per traced triangle */
  /* the same triangles structure-of-arrays, padded to a multiple of
   * ORC_CHUNK with zero triangles (determinant 0 -> never accepted): 9 arrays
   * of n_pad floats {ax ay az e1x e1y e1z e2x e2y e2z} */
  int n_pad;
  float* soa;
} prep_t;

static const float* mesh_tr(const orc_mesh* m, int j, float* tmp) {
  if (m->restricted) {
    orc_restricted_to_mat(m->restricted + 7 * j, tmp);
    return tmp;
  }
  if (m->transforms) return m->transforms + 16 * j;
  mat_identity(tmp);
  return tmp;
}

static f3 ld3(const float* p, int i) { return v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

static void prep_free(prep_t* s) {
  free(s->mesh_block0); free(s->block_off); free(s->block_mesh);
  free(s->pos); free(s->orig); free(s->col); free(s->nrm); free(s->tng); free(s->tc);
  free(s->tr); free(s->tr_inv);
  free(s->tri_block); free(s->tri_prim); free(s->ta); free(s->te1); free(s->te2); free(s->tri_gid);
  free(s->soa);
  memset(s, 0, sizeof(*s));
}

static void prep_build(prep_t* s, const orc_mesh* meshes, int n_meshes) {
  memset(s, 0, sizeof(*s));
  s->meshes = meshes;
  s->n_meshes = n_meshes;
  s->mesh_block0 = (int*)calloc(n_meshes + 1, sizeof(int));
  int nb = 0, total = 0, ntri = 0;
  for (int i = 0; i < n_meshes; i++) {
    s->mesh_block0[i] = nb;
    nb += meshes[i].n_instances;
    total += meshes[i].n_instances * meshes[i].n_vertices;
    ntri += meshes[i].n_instances * (meshes[i].n_indices / 3);
  }
  s->mesh_block0[n_meshes] = nb;
  s->n_blocks = nb;
  s->total = total;
  s->block_off = (int*)calloc(nb, sizeof(int));
  s->block_mesh = (int*)calloc(nb, sizeof(int));
  s->pos = (f3*)calloc(total, sizeof(f3));
  s->orig = (f3*)calloc(total, sizeof(f3));
  s->col = (f3*)calloc(total, sizeof(f3));
  s->nrm = (f3*)calloc(total, sizeof(f3));
  s->tng = (f3*)calloc(total, sizeof(f3));
  s->tc = (f2*)calloc(total, sizeof(f2));
  s->tr = (float*)calloc(16 * nb, sizeof(float));
  s->tr_inv = (float*)calloc(16 * nb, sizeof(float));
  for (int k = 0; k < total; k++) {
    s->nrm[k] = v3(1, 0, 0);
    s->tng[k] = v3(0, 1, 0);
  }
  int off = 0, b = 0;
  for (int i = 0; i < n_meshes; i++) {
    const orc_mesh* m = meshes + i;
    for (int j = 0; j < m->n_instances; j++, b++) {
      float tmp[16], ntr[16], inv[16];
      const float* tr = mesh_tr(m, j, tmp);
      memcpy(s->tr + 16 * b, tr, 16 * sizeof(float));
      mat_inverse(tr, s->tr_inv + 16 * b);
      /* n_tr = transpose(inverse4x4(tr)) */
      mat_inverse(tr, inv);
      for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) M(ntr, r, c) = M(inv, c, r);
      s->block_off[b] = off;
      s->block_mesh[b] = i;
      for (int k = 0; k < m->n_vertices; k++) {
        f3 v = ld3(m->vertices, k);
        s->pos[off + k] = mat_pt(tr, v);
        s->orig[off + k] = v;
        if (m->colors) s->col[off + k] = ld3(m->colors, k);
        if (m->tc) s->tc[off + k] = v2(m->tc[2 * k], m->tc[2 * k + 1]);
        if (m->normals) s->nrm[off + k] = mat_pt(ntr, ld3(m->normals, k));
        if (m->tangents) s->tng[off + k] = mat_pt(ntr, ld3(m->tangents, k));
      }
      off += m->n_vertices;
    }
  }
  s->n_tris = ntri;
  s->tri_block = (int*)calloc(ntri, sizeof(int));
  s->tri_prim = (int*)calloc(ntri, sizeof(int));
  s->ta = (f3*)calloc(ntri, sizeof(f3));
  s->te1 = (f3*)calloc(ntri, sizeof(f3));
  s->te2 = (f3*)calloc(ntri, sizeof(f3));
  s->tri_gid = (int*)calloc(3 * ntri, sizeof(int));
  int t = 0;
  for (b = 0; b < nb; b++) {
    const orc_mesh* m = meshes + s->block_mesh[b];
    const float* tr = s->tr + 16 * b;
    for (int p = 0; p < m->n_indices / 3; p++, t++) {
      int A = s->block_off[b] + (int)m->indices[3 * p + 0];
      int B = s->block_off[b] + (int)m->indices[3 * p + 1];
      int C = s->block_off[b] + (int)m->indices[3 * p + 2];
      f3 Ap = mat_pt(tr, s->pos[A]), Bp = mat_pt(tr, s->pos[B]), Cp = mat_pt(tr, s->pos[C]);
      s->tri_block[t] = b;
      s->tri_prim[t] = p;
      s->ta[t] = Ap;
      s->te1[t] = sub3(Bp, Ap);
      s->te2[t] = sub3(Cp, Ap);
      s->tri_gid[3 * t] = A;
      s->tri_gid[3 * t + 1] = B;
      s->tri_gid[3 * t + 2] = C;
    }
  }
  s->n_pad = (ntri + ORC_CHUNK - 1) / ORC_CHUNK * ORC_CHUNK;
  s->soa = (float*)calloc(9 * (size_t)(s->n_pad > 0 ? s->n_pad : 1), sizeof(float));
  for (t = 0; t < ntri; t++) {
    const f3 q[3] = {s->ta[t], s->te1[t], s->te2[t]};
    for (int k = 0; k < 3; k++) {
      s->soa[(size_t)(3 * k + 0) * s->n_pad + t] = q[k].x;
      s->soa[(size_t)(3 * k + 1) * s->n_pad + t] = q[k].y;
      s->soa[(size_t)(3 * k + 2) * s->n_pad + t] = q[k].z;
    }
  }
}

/* get_index(mesh, inst, k) with the caster's identity instance mapping (scene.h:168-171). */
static inline int get_index(const prep_t* s, int mesh, int inst, int k) {
  return s->block_off[s->mesh_block0[mesh] + inst] + (int)s->meshes[mesh].indices[k];
}

/* ---------------------------------------------------------------------------
 * Brute-force nearest hit (raytrace3d_bf.cpp:102-156) and camera rays
 * (raytrace.h:49-76, raytrace3d_bf.cpp:158-174).
 * ------------------------------------------------------------------------- */
typedef struct { uint32_t prim, inst, geom; float t, u, v; } hit_t;

/* The Moller-Trumbore test of raytrace3d_bf.cpp:127-138 for ORC_CHUNK
 * consecutive triangles: each lane performs the reference's scalar IEEE
 * operations in the reference's order (no contraction), so the values are
 * those of the scalar loop; ok[k] holds every acceptance test except the
 * running `t < best`, which the callers apply in triangle order. */
static inline int mt_chunk(const prep_t* s, int t0, f3 pos, f3 dir, float tNear, float tFar, float* tt, float* uu,
                           float* vv, int* ok) {
  const size_t np = (size_t)s->n_pad;
  const float *ax = s->soa + t0, *ay = ax + np, *az = ay + np;
  const float *e1x = az + np, *e1y = e1x + np, *e1z = e1y + np;
  const float *e2x = e1z + np, *e2y = e2x + np, *e2z = e2y + np;
  int any = 0;
  for (int k = 0; k < ORC_CHUNK; k++) {
    const f3 edge1 = v3(e1x[k], e1y[k], e1z[k]), edge2 = v3(e2x[k], e2y[k], e2z[k]);
    const f3 pvec = cross3(dir, edge2);
    const f3 tvec = sub3(pos, v3(ax[k], ay[k], az[k]));
    const f3 qvec = cross3(tvec, edge1);
    const float e1dpv = dot3(edge1, pvec);
    const float signv = (e1dpv == 0.0f) ? 0.0f : ((e1dpv < 0.0f) ? -1.0f : 1.0f); /* signf_ref */
    const float invDet = signv / maxf_ref(signv * e1dpv, 1e-6f);
    const float v = dot3(tvec, pvec) * invDet;
    const float u = dot3(qvec, dir) * invDet;
    const float t = dot3(edge2, qvec) * invDet;
    const int a = (v > 0.0f) & (u > 0.0f) & (u + v < 1.0f) & (t > tNear) & (t < tFar);
    tt[k] = t;
    uu[k] = u;
    vv[k] = v;
    ok[k] = a;
    any |= a;
  }
  return any;
}

static hit_t nearest_hit(const prep_t* s, f3 pos, f3 dir, float tNear, float tFar) {
  hit_t h = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, tFar, 0.0f, 0.0f};
  float tt[ORC_CHUNK], uu[ORC_CHUNK], vv[ORC_CHUNK];
  int ok[ORC_CHUNK];
  for (int t0 = 0; t0 < s->n_pad; t0 += ORC_CHUNK) {
    if (!mt_chunk(s, t0, pos, dir, tNear, tFar, tt, uu, vv, ok)) continue;
    for (int k = 0; k < ORC_CHUNK; k++) {
      if (ok[k] && tt[k] < h.t) { /* the brute-force loop's order and strict < */
        const int t = t0 + k;
        const int b = s->tri_block[t];
        const int mesh = s->block_mesh[b];
        h.t = tt[k];
        h.geom = (uint32_t)mesh;
        h.inst = (uint32_t)(b - s->mesh_block0[mesh]);
        h.prim = (uint32_t)s->tri_prim[t];
        h.u = uu[k];
        h.v = vv[k];
      }
    }
  }
  return h;
}

/* Whether nearest_hit would report a hit: the first accepted triangle
 * decides, so the scan stops there. */
static int any_hit(const prep_t* s, f3 pos, f3 dir, float tNear, float tFar) {
  float tt[ORC_CHUNK], uu[ORC_CHUNK], vv[ORC_CHUNK];
  int ok[ORC_CHUNK];
  for (int t0 = 0; t0 < s->n_pad; t0 += ORC_CHUNK)
    if (mt_chunk(s, t0, pos, dir, tNear, tFar, tt, uu, vv, ok)) return 1;
  return 0;
}

static void camera_ray(const float* cam, float x, float y, f3* ro, f3* rd) {
  const float* proj_inv = cam + 48;
  const float* wv_inv = cam + 64;
  /* EyeRayDirNormalized(x/w, y/h, ProjInv) */
  const float xn = x / cam[80], yn = y / cam[81];
  float p[4] = {2.0f * xn - 1.0f, -2.0f * yn + 1.0f, 0.0f, 1.0f}, r[4];
  mat_vec4(proj_inv, p, r);
  const float w = r[3];
  r[0] /= w; r[1] /= w; r[2] /= w;
  f3 dir = norm3(v3(r[0], r[1], r[2]));
  /* transform_ray3f */
  f3 pos0 = v3(0, 0, 0);
  f3 pos = mat_pt(wv_inv, pos0);
  f3 pos2 = mat_pt(wv_inv, add3(pos0, scl3(dir, 100.0f)));
  f3 diff = sub3(pos2, pos);
  *ro = pos;
  *rd = norm3(diff);
}

int orc_cast_rays(const orc_mesh* meshes, int n_meshes, const float* cam, const float* xy, int64_t n, uint32_t* prim,
                  uint32_t* inst, uint32_t* geom, float* t, float* u, float* v, float* ray_pos, float* ray_dir) {
  prep_t s;
  prep_build(&s, meshes, n_meshes);
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
  for (int64_t i = 0; i < n; i++) {
    f3 ro, rd;
    camera_ray(cam, xy[2 * i], xy[2 * i + 1], &ro, &rd);
    hit_t h = nearest_hit(&s, ro, rd, 0.0f, 1e9f);
    prim[i] = h.prim; inst[i] = h.inst; geom[i] = h.geom;
    t[i] = h.t; u[i] = h.u; v[i] = h.v;
    if (ray_pos) { ray_pos[3 * i] = ro.x; ray_pos[3 * i + 1] = ro.y; ray_pos[3 * i + 2] = ro.z; }
    if (ray_dir) { ray_dir[3 * i] = rd.x; ray_dir[3 * i + 1] = rd.y; ray_dir[3 * i + 2] = rd.z; }
  }
  prep_free(&s);
  return 0;
}

/* ---------------------------------------------------------------------------
 * Shading models (src/shade_simple.cpp, src/shade_lambert.cpp,
 * src/shade_common.cpp) and the two models without a reference counterpart.
 * ------------------------------------------------------------------------- */
void orc_default_model_params(orc_model_params* p) {
  p->light_pos[0] = 3.0f; p->light_pos[1] = 3.0f; p->light_pos[2] = 3.0f;
  p->light_intensity = 10.0f;
  p->ambient = 0.1f;
  p->path_depth = 2;
  p->seed = 1u;
  p->edge_jacobian = 0;
  p->edge_set = 0;
}

/* sample_bilinear_clamp_3f, shade_common.cpp:3-21 */
static f3 sample_bilinear(f2 tc, int w, int h, const float* data) {
  tc.x = clampf_ref(tc.x, 0.0f, 1.0f);
  tc.y = clampf_ref(tc.y, 0.0f, 1.0f);
  tc.x *= (float)w;
  tc.y *= (float)h;
  const int ix = (int)tc.x, iy = (int)tc.y;
  const int x0 = clampi(ix, 0, w - 1), y0 = clampi(iy, 0, h - 1);
  const int x1 = clampi(ix + 1, 0, w - 1), y1 = clampi(iy + 1, 0, h - 1);
  const float dx = tc.x - (float)x0, dy = tc.y - (float)y0;
  const float* p00 = data + 3 * (y0 * w + x0);
  const float* p01 = data + 3 * (y1 * w + x0);
  const float* p10 = data + 3 * (y0 * w + x1);
  const float* p11 = data + 3 * (y1 * w + x1);
  float r[3];
  for (int i = 0; i < 3; i++)
    r[i] = (1 - dx) * (1 - dy) * p00[i] + (1 - dx) * dy * p01[i] + dx * (1 - dy) * p10[i] + dx * dy * p11[i];
  return v3(r[0], r[1], r[2]);
}

/* sample_bilinear_clamp_3f_grad, shade_common.cpp:23-46 (no clamp of tc) */
static void sample_bilinear_grad(f3 val, f2 tc, int w, int h, float* data) {
  const float px = tc.x * (float)w, py = tc.y * (float)h;
  const int ix = (int)px, iy = (int)py;
  const int x0 = clampi(ix, 0, w - 1), y0 = clampi(iy, 0, h - 1);
  const int x1 = clampi(ix + 1, 0, w - 1), y1 = clampi(iy + 1, 0, h - 1);
  const float dx = px - (float)x0, dy = py - (float)y0;
  float* d00 = data + 3 * (y0 * w + x0);
  float* d01 = data + 3 * (y1 * w + x0);
  float* d10 = data + 3 * (y0 * w + x1);
  float* d11 = data + 3 * (y1 * w + x1);
  d00[0] += (1 - dx) * (1 - dy) * val.x; d00[1] += (1 - dx) * (1 - dy) * val.y; d00[2] += (1 - dx) * (1 - dy) * val.z;
  d01[0] += (1 - dx) * dy * val.x;       d01[1] += (1 - dx) * dy * val.y;       d01[2] += (1 - dx) * dy * val.z;
  d10[0] += dx * (1 - dy) * val.x;       d10[1] += dx * (1 - dy) * val.y;       d10[2] += dx * (1 - dy) * val.z;
  d11[0] += dx * dy * val.x;             d11[1] += dx * dy * val.y;             d11[2] += dx * dy * val.z;
}

/* barycentric interpolation in the reference's form: a*(1-u-v) + b*v + u*c */
static inline f3 interp3(f3 a, f3 b, f3 c, float u, float v) {
  const float w0 = 1.0f - u - v;
  return add3(add3(scl3(a, w0), scl3(b, v)), scl3(c, u));
}
static inline f2 interp2(f2 a, f2 b, f2 c, float u, float v) {
  const float w0 = 1.0f - u - v;
  return add2(add2(scl2(a, w0), scl2(b, v)), scl2(c, u));
}

typedef struct {
  const prep_t* s;
  const float* cam;
  int mode;
  const orc_model_params* mp;
} ctx_t;

/* Counter-based hash for the path model (no reference counterpart). */
static inline uint32_t pcg_hash(uint32_t x) {
  uint32_t state = x * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}
static inline float rnd01(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t h = pcg_hash(a ^ pcg_hash(b ^ pcg_hash(c)));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

/* Hit information shared by shade and shade_grad. */
typedef struct {
  hit_t h;
  int A, B, C; /* global vertex ids */
  f3 ro, rd;
} surf_t;

static int cast(const ctx_t* c, f2 sp, surf_t* out) {
  camera_ray(c->cam, sp.x, sp.y, &out->ro, &out->rd);
  out->h = nearest_hit(c->s, out->ro, out->rd, 0.0f, 1e9f);
  if (out->h.prim == 0xFFFFFFFFu) return 0;
  out->A = get_index(c->s, (int)out->h.geom, (int)out->h.inst, (int)out->h.prim * 3 + 0);
  out->B = get_index(c->s, (int)out->h.geom, (int)out->h.inst, (int)out->h.prim * 3 + 1);
  out->C = get_index(c->s, (int)out->h.geom, (int)out->h.inst, (int)out->h.prim * 3 + 2);
  return 1;
}

/* Lighting factor of the point-light vertex-albedo model: vis*I*max(0,n.l)/d2 + ambient. */
static float lpv_factor(const ctx_t* c, const surf_t* sf) {
  const prep_t* s = c->s;
  const float u = sf->h.u, v = sf->h.v;
  const f3 n = interp3(s->nrm[sf->A], s->nrm[sf->B], s->nrm[sf->C], u, v);
  const f3 p = add3(sf->ro, scl3(sf->rd, sf->h.t - 1e-5f));
  const f3 L = sub3(v3(c->mp->light_pos[0], c->mp->light_pos[1], c->mp->light_pos[2]), p);
  const float d2 = dot3(L, L);
  const float dist = sqrtf(d2);
  const f3 l = div3s(L, dist);
  const float ndl = maxf_ref(0.0f, dot3(n, l));
  /* the lit term is 0 when n.l <= 0 whatever the visibility */
  const float vis = (ndl > 0.0f && any_hit(s, p, l, 0.0f, dist)) ? 0.0f : 1.0f;
  return vis * c->mp->light_intensity * ndl / d2 + c->mp->ambient;
}

/* sin and cos of 2*pi*x, x in [0, 1): exact quadrant split (x*4, its nearest
 * integer q and 4x - q are exact), Taylor series of sin to a^9 and cos to
 * a^10 on a = (4x - q)*pi/2 in [-pi/4, pi/4] (error < 2e-9), rotated by the
 * quadrant.  The CUDA path evaluates the same operations in the same order,
 * so the bounce directions are bit-identical on both sides. */
static void sincos_small(float a, float* ps, float* pc) {
  const float a2 = a * a;
  *ps = a * (1.0f + a2 * (-1.66666672e-1f + a2 * (8.33333377e-3f + a2 * (-1.98412701e-4f + a2 * 2.75573188e-6f))));
  *pc = 1.0f + a2 * (-0.5f + a2 * (4.16666679e-2f + a2 * (-1.38888892e-3f + a2 * (2.48015876e-5f +
                                                                                a2 * -2.75573188e-7f))));
}
static void sincos_turns(float x, float* s, float* c) {
  const float x4 = x * 4.0f;
  const float q = rintf(x4);
  float ps, pc;
  sincos_small((x4 - q) * 1.57079633f, &ps, &pc);
  switch (((int)q) & 3) {
    case 0: *s = ps; *c = pc; break;
    case 1: *s = pc; *c = -ps; break;
    case 2: *s = -ps; *c = -pc; break;
    default: *s = -pc; *c = ps; break;
  }
}

/* Fixed-depth diffuse path tracer (no reference counterpart; structure of
 * shade<PATH_TEST>, shade_path_test.cpp:232-282, with a counter-based RNG
 * and `path_depth` bounces).  Returns radiance and the albedo-weighted
 * throughput of the primary vertex (its derivative w.r.t. the primary
 * albedo divided by that albedo). */
static f3 path_diffuse(const ctx_t* c, const surf_t* first, uint32_t sample_key, f3* d_albedo0) {
  const prep_t* s = c->s;
  const f3 lp = v3(c->mp->light_pos[0], c->mp->light_pos[1], c->mp->light_pos[2]);
  const float I = c->mp->light_intensity;
  f3 L = v3(0, 0, 0), beta = v3(1, 1, 1);
  f3 beta_noalb0 = v3(1, 1, 1);
  f3 dL0 = v3(0, 0, 0);
  surf_t sf = *first;
  f3 ro = first->ro, rd = first->rd;
  for (int bounce = 0; bounce <= c->mp->path_depth; bounce++) {
    if (bounce > 0) {
      sf.h = nearest_hit(s, ro, rd, 0.0f, 1e9f);
      if (sf.h.prim == 0xFFFFFFFFu) {
        L = add3(L, scl3(beta, c->mp->ambient));
        dL0 = add3(dL0, scl3(beta_noalb0, c->mp->ambient));
        break;
      }
      sf.A = get_index(s, (int)sf.h.geom, (int)sf.h.inst, (int)sf.h.prim * 3 + 0);
      sf.B = get_index(s, (int)sf.h.geom, (int)sf.h.inst, (int)sf.h.prim * 3 + 1);
      sf.C = get_index(s, (int)sf.h.geom, (int)sf.h.inst, (int)sf.h.prim * 3 + 2);
    }
    const float u = sf.h.u, v = sf.h.v;
    const f3 alb = interp3(s->col[sf.A], s->col[sf.B], s->col[sf.C], u, v);
    f3 n = norm3(interp3(s->nrm[sf.A], s->nrm[sf.B], s->nrm[sf.C], u, v));
    const f3 ng = norm3(cross3(sub3(s->pos[sf.B], s->pos[sf.A]), sub3(s->pos[sf.C], s->pos[sf.A])));
    if (dot3(ng, rd) > 0.0f) n = scl3(n, -1.0f);
    const f3 ngf = dot3(ng, n) < 0.0f ? scl3(ng, -1.0f) : ng;
    const f3 p = add3(add3(ro, scl3(rd, sf.h.t)), scl3(ngf, 1e-4f));
    /* direct light: point light, Lambert BRDF albedo/pi */
    const f3 Lv = sub3(lp, p);
    const float d2 = dot3(Lv, Lv);
    const float dist = sqrtf(d2);
    const f3 l = div3s(Lv, dist);
    const float ndl = maxf_ref(0.0f, dot3(n, l));
    if (ndl > 0.0f && !any_hit(s, p, l, 0.0f, dist)) {
      const float k = I * ndl / (d2 * 3.14159265f);
      L = add3(L, scl3(mul3(beta, alb), k));
      dL0 = add3(dL0, scl3(bounce == 0 ? beta_noalb0 : mul3(beta_noalb0, alb), k));
    }
    if (bounce == c->mp->path_depth) break;
    /* cosine-weighted bounce: throughput *= albedo (pdf cancels cos/pi) */
    const float r1 = rnd01(sample_key, (uint32_t)bounce, c->mp->seed);
    const float r2 = rnd01(sample_key, (uint32_t)bounce + 1000u, c->mp->seed);
    float sphi, cphi;
    sincos_turns(r1, &sphi, &cphi); /* azimuth 2*pi*r1 */
    const float sr = sqrtf(r2);
    const f3 a = fabsf(n.x) > 0.5f ? v3(0, 1, 0) : v3(1, 0, 0);
    const f3 ex = norm3(cross3(a, n));
    const f3 ey = cross3(n, ex);
    const float lx = sr * cphi, ly = sr * sphi, lz = sqrtf(maxf_ref(0.0f, 1.0f - r2));
    rd = norm3(add3(add3(scl3(ex, lx), scl3(ey, ly)), scl3(n, lz)));
    ro = p;
    beta_noalb0 = bounce == 0 ? beta_noalb0 : mul3(beta_noalb0, alb);
    beta = mul3(beta, alb);
  }
  if (d_albedo0) *d_albedo0 = dL0;
  return L;
}

/* ConcentricSampleDisk, shade_path_test.cpp:77-95 (Shirley and Chiu's
 * concentric map): the angle of either wedge reduced to [-pi/4, pi/4]
 * (cos(pi/2 - b) = sin b, sin(pi/2 - b) = cos b) for sincos_small. */
static f2 concentric_disk(float u0, float u1) {
  const float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
  float sn, cs;
  if (ox == 0.0f && oy == 0.0f) return v2(0.0f, 0.0f);
  if (fabsf(ox) > fabsf(oy)) {
    sincos_small(0.785398163f * (oy / ox), &sn, &cs);
    return v2(ox * cs, ox * sn);
  }
  sincos_small(0.785398163f * (ox / oy), &sn, &cs);
  return v2(oy * sn, oy * cs);
}

/* intensity(), shade_path_test.cpp:75 (double weights) */
static float path_luminance(f3 c) { return (float)(0.2126 * (double)c.x + 0.7152 * (double)c.y + 0.0722 * (double)c.z); }

/* shade<PATH_TEST>, shade_path_test.cpp:133-282: at most MAX_DEPTH = 8
 * bounces, Russian roulette for bounce > RR_DEPTH = 3, get_extended_surface_info
 * (interpolated unnormalised normal n, tangent frame e_x = normalize(n x t),
 * e_y = normalize(n x e_x), n_geom, position offset 1e-4 n_geom, texture
 * albedo), direct_light/sample_light (light colour normalize(1,0.8,0.5)
 * (scene.h:77-82) x 2 at (0,0.7,0.7)
 * + 0.1 * [-1,1]^3, visibility = no hit on the whole line toward it),
 * bsdf_sample_f_diffuse (cosine sample, flipped to wo's side, pdf |cos|/pi
 * or 1e9), ambient 0.5 on leaving the scene.  The reference's rand() is
 * replaced by rnd01(key, 8*bounce + j, seed): j = 0..2 light jitter, 3..4
 * bounce direction, 5 roulette.  A path whose throughput is exactly zero
 * stops (all its further terms are zero). */
static f3 path_test(const ctx_t* c, const surf_t* first, uint32_t key) {
  const prep_t* s = c->s;
  const float PI_F = 3.14159265358979323846f;
  const uint32_t seed = c->mp->seed;
  f3 L = v3(0, 0, 0), beta = v3(1, 1, 1);
  surf_t sf = *first;
  f3 ro = first->ro, rd = first->rd;
  for (int bounce = 0; bounce < 8; bounce++) {
    if (bounce > 0) {
      sf.h = nearest_hit(s, ro, rd, 0.0f, 1e9f);
      if (sf.h.prim == 0xFFFFFFFFu) {
        L = add3(L, scl3(beta, 0.5f));
        break;
      }
      sf.A = get_index(s, (int)sf.h.geom, (int)sf.h.inst, (int)sf.h.prim * 3 + 0);
      sf.B = get_index(s, (int)sf.h.geom, (int)sf.h.inst, (int)sf.h.prim * 3 + 1);
      sf.C = get_index(s, (int)sf.h.geom, (int)sf.h.inst, (int)sf.h.prim * 3 + 2);
    }
    const uint32_t r0 = 8u * (uint32_t)bounce;
    const float u = sf.h.u, v = sf.h.v;
    const orc_mesh* m = s->meshes + sf.h.geom;
    const f2 tc = interp2(s->tc[sf.A], s->tc[sf.B], s->tc[sf.C], u, v);
    const f3 n = interp3(s->nrm[sf.A], s->nrm[sf.B], s->nrm[sf.C], u, v);
    const f3 tg = interp3(s->tng[sf.A], s->tng[sf.B], s->tng[sf.C], u, v);
    const f3 ng = norm3(cross3(sub3(s->pos[sf.B], s->pos[sf.A]), sub3(s->pos[sf.C], s->pos[sf.A])));
    const f3 p = add3(add3(ro, scl3(rd, sf.h.t)), scl3(ng, 1e-4f));
    const f3 ex = norm3(cross3(n, tg));
    const f3 ey = norm3(cross3(n, ex));
    const f3 alb = sample_bilinear(tc, m->tex_w, m->tex_h, m->texture);
    /* direct light */
    const f3 jit = v3(2.0f * rnd01(key, r0, seed) - 1.0f, 2.0f * rnd01(key, r0 + 1u, seed) - 1.0f,
                      2.0f * rnd01(key, r0 + 2u, seed) - 1.0f);
    const f3 lv = sub3(add3(v3(0.0f, 0.7f, 0.7f), scl3(jit, 0.1f)), p);
    const float ld = dot3(lv, lv);
    const f3 l = div3s(lv, sqrtf(ld));
    if (!any_hit(s, p, l, 0.0f, 1e9f)) {
      const f3 Li = div3s(scl3(norm3(v3(1.0f, 0.8f, 0.5f)), 2.0f), ld); /* PointLight normalises its colour */
      L = add3(L, mul3(beta, mul3(Li, scl3(div3s(alb, PI_F), maxf_ref(0.0f, dot3(n, l))))));
    }
    /* next direction */
    const f3 wo = norm3(scl3(rd, -1.0f));
    const float woz = dot3(wo, n);
    const f2 d = concentric_disk(rnd01(key, r0 + 3u, seed), rnd01(key, r0 + 4u, seed));
    float wz = sqrtf(maxf_ref(0.0f, 1.0f - d.x * d.x - d.y * d.y));
    if (woz < 0.0f) wz = -wz;
    const float pdf = woz * wz > 0.0f ? fabsf(wz) / PI_F : 1e9f;
    const f3 nd = v3(ex.x * d.x + ey.x * d.y + n.x * wz, ex.y * d.x + ey.y * d.y + n.y * wz,
                     ex.z * d.x + ey.z * d.y + n.z * wz);
    beta = mul3(beta, div3s(scl3(div3s(alb, PI_F), maxf_ref(0.0f, dot3(ng, nd))), pdf));
    rd = nd;
    ro = p;
    if (bounce > 3) {
      const float q = maxf_ref(0.05f, 1.0f - path_luminance(beta));
      if (rnd01(key, r0 + 5u, seed) < q) break;
      beta = div3s(beta, 1.0f - q);
    }
    if (beta.x == 0.0f && beta.y == 0.0f && beta.z == 0.0f) break;
  }
  return L;
}

static f3 shade(const ctx_t* c, f2 sp) {
  surf_t sf;
  const prep_t* s = c->s;
  if (!cast(c, sp, &sf)) {
    if (c->mode == ORC_PATH_DIFFUSE) return v3(c->mp->ambient, c->mp->ambient, c->mp->ambient);
    return v3(0, 0, 0);
  }
  const float u = sf.h.u, v = sf.h.v;
  switch (c->mode) {
    case ORC_SILHOUETTE: /* shade_simple.cpp:7-14 */
      return v3(1, 1, 1);
    case ORC_VERTEX_COLOR: /* shade_simple.cpp:24-37 */
      return interp3(s->col[sf.A], s->col[sf.B], s->col[sf.C], u, v);
    case ORC_TEXTURE_COLOR: { /* shade_simple.cpp:114-130 */
      const orc_mesh* m = s->meshes + sf.h.geom;
      f2 tc = interp2(s->tc[sf.A], s->tc[sf.B], s->tc[sf.C], u, v);
      return sample_bilinear(tc, m->tex_w, m->tex_h, m->texture);
    }
    case ORC_LAMBERT: { /* shade_lambert.cpp:7-35 */
      const f3 light_dir = norm3(v3(-1, -1, 0));
      const f3 light_color = v3(1.0f, 0.5f, 0.2f);
      const f3 ambient = scl3(v3(1, 1, 1), 0.1f);
      const float BIAS = 1e-5f;
      const orc_mesh* m = s->meshes + sf.h.geom;
      f2 tc = interp2(s->tc[sf.A], s->tc[sf.B], s->tc[sf.C], u, v);
      f3 n = interp3(s->nrm[sf.A], s->nrm[sf.B], s->nrm[sf.C], u, v);
      f3 diffuse = sample_bilinear(tc, m->tex_w, m->tex_h, m->texture);
      f3 surf_pos = add3(sf.ro, scl3(sf.rd, sf.h.t - BIAS));
      const f3 to_light = scl3(light_dir, -1.0f);
      const float ndl = maxf_ref(0.0f, dot3(n, to_light));
      /* (colour * vis) * 0 is 0 for either visibility: trace only when lit */
      float sh = (ndl > 0.0f && any_hit(s, surf_pos, to_light, 0.0f, 1e9f)) ? 0.0f : 1.0f;
      f3 lit = scl3(scl3(light_color, sh), ndl);
      return mul3(add3(lit, ambient), diffuse);
    }
    case ORC_PHONG:   /* shade_lambert.cpp:45-77 */
    case ORC_GGX: {   /* shade_lambert.cpp:128-161 */
      const int phong = c->mode == ORC_PHONG;
      const f3 light_dir = phong ? norm3(v3(0.0f, -0.25f, -1.0f)) : norm3(v3(0.15f, 0.0f, -1.0f));
      const f3 light_color = v3(1.0f, 0.5f, 0.2f);
      const float Ka = phong ? 0.1f : 0.01f;
      const float BIAS = 1e-5f;
      const orc_mesh* m = s->meshes + sf.h.geom;
      f2 tc = interp2(s->tc[sf.A], s->tc[sf.B], s->tc[sf.C], u, v);
      f3 n = interp3(s->nrm[sf.A], s->nrm[sf.B], s->nrm[sf.C], u, v);
      f3 diffuse = sample_bilinear(tc, m->tex_w, m->tex_h, m->texture);
      f3 surf_pos = add3(sf.ro, scl3(sf.rd, sf.h.t - BIAS));
      const f3 to_light = scl3(light_dir, -1.0f);
      float term;
      if (phong) {
        /* Kd*max(0,n.-L) + Ks*pow(max(0,n.r),32); the reference's pow(float,int)
         * is pow(double,double), so the sum is a double */
        const float ndl = maxf_ref(0.0f, dot3(n, to_light));
        const f3 refl = sub3(light_dir, scl3(n, 2.0f * dot3(n, light_dir)));
        const double spec = pow((double)maxf_ref(0.0f, dot3(n, refl)), 32.0);
        term = (float)((double)(1.0f * ndl) + (double)1.0f * spec);
      } else {
        /* LightingFuncGGX(n, -view, -light, 0.2, 0.8), shade_lambert.cpp:90-124 */
        const f3 N = n, V = scl3(sf.rd, -1.0f), L = to_light;
        const float roughness = 0.2f, F0 = 0.8f;
        const float alpha = roughness * roughness;
        const f3 H = norm3(add3(V, L));
        const float dotNL = maxf_ref(0.0f, minf_ref(1.0f, dot3(N, L)));
        const float dotNV = maxf_ref(0.0f, minf_ref(1.0f, dot3(N, V)));
        const float dotNH = maxf_ref(0.0f, minf_ref(1.0f, dot3(N, H)));
        const float dotLH = maxf_ref(0.0f, minf_ref(1.0f, dot3(L, H)));
        const float alphaSqr = alpha * alpha;
        const float pi = 3.14159f;
        const float denom = (float)((double)(dotNH * dotNH) * ((double)alphaSqr - 1.0) + 1.0);
        const float D = alphaSqr / (pi * denom * denom);
        const float dotLH5 = (float)pow((double)(1.0f - dotLH), 5.0);
        const float F = (float)((double)F0 + (1.0 - (double)F0) * (double)dotLH5);
        const float k = alpha / 2.0f;
        const float vis = (1.0f / (dotNL * (1.0f - k) + k)) * (1.0f / (dotNV * (1.0f - k) + k));
        const float ggx = dotNL * D * F * vis;
        term = maxf_ref(0.0f, dot3(n, to_light)) + ggx;
      }
      /* (colour * vis) * 0 is 0 for either visibility: trace only when lit */
      const float sh = (term != 0.0f && any_hit(s, surf_pos, to_light, 0.0f, 1e9f)) ? 0.0f : 1.0f;
      const f3 lit = scl3(scl3(light_color, sh), term);
      return mul3(add3(lit, scl3(v3(1, 1, 1), Ka)), diffuse);
    }
    case ORC_LAMBERT_POINT_VCOLOR: {
      const f3 alb = interp3(s->col[sf.A], s->col[sf.B], s->col[sf.C], u, v);
      return scl3(alb, lpv_factor(c, &sf));
    }
    case ORC_PATH_DIFFUSE: {
      /* the sample key is folded into sp by the caller through the RNG key */
      return v3(0, 0, 0);
    }
    default:
      return v3(0, 0, 0);
  }
}

/* ---------------------------------------------------------------------------
 * Gradient layout (DMesh, dmesh.h:35-85).
 * ------------------------------------------------------------------------- */
typedef struct {
  int vertices, instances, pos_off, color_off, tex_off, tr_off, rt_off, full;
} dlayout_t;

static int mode_has_color(int mode) { return mode == ORC_VERTEX_COLOR || mode == ORC_LAMBERT_POINT_VCOLOR || mode == ORC_PATH_DIFFUSE; }
static int mode_has_tex(int mode) {
  return mode == ORC_TEXTURE_COLOR || mode == ORC_LAMBERT || mode == ORC_PHONG || mode == ORC_GGX ||
         mode == ORC_PATH_TEST;
}

static dlayout_t make_layout(const orc_mesh* m, int mode) {
  dlayout_t L;
  int tex = (mode_has_tex(mode) && m->texture) ? m->tex_w * m->tex_h * m->tex_channels : 0;
  L.vertices = m->n_vertices;
  L.instances = m->n_instances;
  int off = 0;
  L.pos_off = off; off += 3 * m->n_vertices;
  L.color_off = -1;
  if (mode_has_color(mode)) { L.color_off = off; off += 3 * m->n_vertices; }
  L.tex_off = -1;
  if (mode_has_tex(mode) && m->texture) { L.tex_off = off; off += tex; }
  /* transform matrices, or the restricted parameters (dmesh.h:42-50,76-84) */
  L.tr_off = L.rt_off = -1;
  if (m->restricted) { L.rt_off = off; off += 7 * m->n_instances; }
  else { L.tr_off = off; off += 12 * m->n_instances; }
  L.full = off;
  return L;
}

int orc_dscene_layout(const orc_mesh* meshes, int n_meshes, int mode, const int32_t* ids, int n_ids, int32_t* layout,
                      int64_t* total) {
  int64_t t = 0;
  for (int k = 0; k < n_ids; k++) {
    if (ids[k] < 0 || ids[k] >= n_meshes) return -1;
    dlayout_t L = make_layout(meshes + ids[k], mode);
    int32_t* o = layout + 9 * k;
    o[0] = L.vertices; o[1] = L.instances; o[2] = L.pos_off; o[3] = L.color_off; o[4] = L.tex_off;
    o[5] = L.tr_off; o[6] = L.rt_off; o[7] = L.full; o[8] = ids[k];
    t += L.full;
  }
  if (total) *total = t;
  return 0;
}

typedef struct {
  int n;             /* number of differentiable meshes */
  int ids[16];
  dlayout_t lay[16];
  int64_t base[16];  /* offset of each DMesh block in the flat vector */
  int64_t total;
  int by_mesh[64];   /* mesh id -> dmesh slot, -1 if not differentiable */
} dmap_t;

static int dmap_build(dmap_t* d, const orc_mesh* meshes, int n_meshes, int mode, const int32_t* ids, int n_ids) {
  if (n_ids > 16 || n_meshes > 64) return -1;
  memset(d, 0, sizeof(*d));
  for (int i = 0; i < 64; i++) d->by_mesh[i] = -1;
  d->n = n_ids;
  int64_t off = 0;
  for (int k = 0; k < n_ids; k++) {
    if (ids[k] < 0 || ids[k] >= n_meshes) return -1;
    d->ids[k] = ids[k];
    d->lay[k] = make_layout(meshes + ids[k], mode);
    d->base[k] = off;
    off += d->lay[k].full;
    d->by_mesh[ids[k]] = k;
  }
  d->total = off;
  return 0;
}

/* libgomp static schedule: block k of n iterations over T threads. */
static void static_block(int64_t n, int T, int k, int64_t* b, int64_t* e) {
  int64_t q = n / T, r = n % T;
  if (k < r) { q++; r = 0; }
  *b = q * k + r;
  *e = *b + q;
}

/* ---------------------------------------------------------------------------
 * Forward render (drender.h:98-141).
 * ------------------------------------------------------------------------- */
static f3 shade_sample(const ctx_t* c, f2 sp, uint32_t key) {
  surf_t sf;
  if (c->mode == ORC_PATH_TEST) {
    if (!cast(c, sp, &sf)) return v3(0.5f, 0.5f, 0.5f);
    return path_test(c, &sf, key);
  }
  if (c->mode != ORC_PATH_DIFFUSE) return shade(c, sp);
  if (!cast(c, sp, &sf)) return v3(c->mp->ambient, c->mp->ambient, c->mp->ambient);
  return path_diffuse(c, &sf, key, NULL);
}

static void render_view(const prep_t* s, int mode, int spp, const orc_model_params* mp, const float* cam, float* img,
                        uint32_t view_key) {
  const int W = (int)cam[80], H = (int)cam[81];
  const int sq = (int)sqrtf((float)spp);
  const int S = sq * sq;
  ctx_t c = {s, cam, mode, mp};
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
  for (int y = 0; y < H; y++) {
    for (int x = 0; x < W; x++) {
      f3 acc = v3(0, 0, 0);
      for (int dy = 0; dy < sq; dy++)
        for (int dx = 0; dx < sq; dx++) {
          const float xoff = (dx + 0.5f) / (float)sq;
          const float yoff = (dy + 0.5f) / (float)sq;
          const f2 sp = v2((float)x + xoff, (float)y + yoff);
          const uint32_t key = view_key ^ (uint32_t)(((y * W + x) * 64 + dy * sq + dx) * 2654435761u);
          const f3 col = shade_sample(&c, sp, key);
          acc = add3(acc, div3s(col, (float)S));
        }
      float* o = img + 3 * ((int64_t)y * W + x);
      o[0] = acc.x; o[1] = acc.y; o[2] = acc.z;
    }
  }
}

int orc_render(const orc_mesh* meshes, int n_meshes, int mode, int spp, const orc_model_params* mp, const float* cams,
               int n_views, float* images) {
  orc_model_params dmp;
  if (!mp) { orc_default_model_params(&dmp); mp = &dmp; }
  prep_t s;
  prep_build(&s, meshes, n_meshes);
  int64_t off = 0;
  for (int vi = 0; vi < n_views; vi++) {
    const float* cam = cams + ORC_CAM_FLOATS * vi;
    render_view(&s, mode, spp, mp, cam, images + off, (uint32_t)vi * 0x9E3779B9u);
    off += 3 * (int64_t)cam[80] * (int64_t)cam[81];
  }
  prep_free(&s);
  return 0;
}

/* ---------------------------------------------------------------------------
 * Interior derivatives (drender.h:197-233) with shade_grad<M>
 * (shade_simple.cpp:40-111, 133-162; shade_lambert.cpp:38-42).
 * ------------------------------------------------------------------------- */
static void shade_grad(const ctx_t* c, const dmap_t* dm, f2 sp, f3 val, float* grad, uint32_t key) {
  const prep_t* s = c->s;
  surf_t sf;
  if (!cast(c, sp, &sf)) return;
  const int slot = dm->by_mesh[sf.h.geom];
  if (slot < 0) return;
  float* g = grad + dm->base[slot];
  const dlayout_t* L = dm->lay + slot;
  const orc_mesh* m = s->meshes + sf.h.geom;
  const float u = sf.h.u, v = sf.h.v;
  if (c->mode == ORC_VERTEX_COLOR || c->mode == ORC_LAMBERT_POINT_VCOLOR || c->mode == ORC_PATH_DIFFUSE) {
    /* get_vertex_n: mesh-local vertex ids */
    const int A = (int)m->indices[sf.h.prim * 3 + 0];
    const int B = (int)m->indices[sf.h.prim * 3 + 1];
    const int C = (int)m->indices[sf.h.prim * 3 + 2];
    f3 ca, cb, cc;
    if (c->mode == ORC_VERTEX_COLOR) {
      ca = scl3(val, 1.0f - u - v);
      cb = scl3(val, v);
      cc = scl3(val, u);
    } else if (c->mode == ORC_LAMBERT_POINT_VCOLOR) {
      const float k = lpv_factor(c, &sf);
      ca = scl3(val, (1.0f - u - v) * k);
      cb = scl3(val, v * k);
      cc = scl3(val, u * k);
    } else {
      f3 d0;
      path_diffuse(c, &sf, key, &d0);
      const f3 vd = mul3(val, d0);
      ca = scl3(vd, 1.0f - u - v);
      cb = scl3(vd, v);
      cc = scl3(vd, u);
    }
    float* col = g + L->color_off;
    col[3 * A + 0] += ca.x; col[3 * A + 1] += ca.y; col[3 * A + 2] += ca.z;
    col[3 * B + 0] += cb.x; col[3 * B + 1] += cb.y; col[3 * B + 2] += cb.z;
    col[3 * C + 0] += cc.x; col[3 * C + 1] += cc.y; col[3 * C + 2] += cc.z;
  } else if (mode_has_tex(c->mode)) { /* PHONG, GGX: shade_lambert.cpp:80-84, 163-168; PATH_TEST: shade_path_test.cpp:284-289 */
    if (L->tex_off < 0) return;
    const f2 tc = interp2(s->tc[sf.A], s->tc[sf.B], s->tc[sf.C], u, v);
    sample_bilinear_grad(val, tc, m->tex_w, m->tex_h, g + L->tex_off);
  }
}

static void interior_derivatives(const prep_t* s, const dmap_t* dm, int mode, int spp, const orc_model_params* mp,
                                 const float* cam, const float* adj, float* dscene, uint32_t view_key) {
  const int W = (int)cam[80], H = (int)cam[81];
  const int sq = (int)sqrtf((float)spp);
  const int S = sq * sq;
  float* ham = (float*)malloc(sizeof(float) * 2 * (spp > 0 ? spp : 1));
  orc_hammersley(spp, ham);
  ctx_t c = {s, cam, mode, mp};
  float* part = (float*)calloc((size_t)REF_THREADS * dm->total, sizeof(float));
  const int64_t n = (int64_t)W * H;
#pragma omp parallel for schedule(dynamic, 1) num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
  for (int k = 0; k < REF_THREADS; k++) {
    int64_t b, e;
    static_block(n, REF_THREADS, k, &b, &e);
    float* g = part + (int64_t)k * dm->total;
    for (int64_t i = b; i < e; i++) {
      const int y = (int)(i / W), x = (int)(i % W);
      const float* a = adj + 3 * i;
      for (int sam = 0; sam < S; sam++) {
        const float xoff = ham[2 * sam + 0], yoff = ham[2 * sam + 1];
        const f3 val = div3s(v3(a[0], a[1], a[2]), (float)S);
        const uint32_t key = view_key ^ 0x5bd1e995u ^ (uint32_t)((i * 64 + sam) * 2654435761u);
        shade_grad(&c, dm, v2((float)x + xoff, (float)y + yoff), val, g, key);
      }
    }
  }
  for (int k = 0; k < REF_THREADS; k++)
    for (int64_t j = 0; j < dm->total; j++) dscene[j] += part[(int64_t)k * dm->total + j];
  free(part);
  free(ham);
}

/* ---------------------------------------------------------------------------
 * Edge sampling (drender.h:235-425, drender.cpp:5-87, functions.cpp:21-163).
 * ------------------------------------------------------------------------- */
typedef struct { int v0, v1, vn0, vn1, mesh, inst, tri0, tri1; } edge_t; /* tri0/1: adjacent traced triangles (-1: none) */

static int edge_cmp(const void* a, const void* b) {
  const edge_t* x = (const edge_t*)a;
  const edge_t* y = (const edge_t*)b;
  if (x->v0 != y->v0) return x->v0 < y->v0 ? -1 : 1;
  if (x->v1 != y->v1) return x->v1 < y->v1 ? -1 : 1;
  return 0;
}

/* VertexShader, functions.h:5-13 */
static void vertex_shader(const float* cam, float vx, float vy, float vz, float out[2]) {
  const float* m = cam + 32;
  const float W = vx * m[3] + vy * m[7] + vz * m[11] + m[15];
  const float xNDC = (vx * m[0] + vy * m[4] + vz * m[8] + m[12]) / W;
  const float yNDC = -(vx * m[1] + vy * m[5] + vz * m[9] + m[13]) / W;
  out[0] = (xNDC * 0.5f + 0.5f) * cam[80];
  out[1] = (yNDC * 0.5f + 0.5f) * cam[81];
}

/* VS_X_grad / VS_Y_grad, functions.cpp:21-163 (reverse-mode derivative of the
 * projected x or y w.r.t. the world vertex, evaluated in the same order). */
static void vs_grad(const float* cam, f3 V, int which_y, float d[3]) {
  const float* m = cam + 32;
  const float t1 = V.x, t0 = m[3], t3 = V.y, t2 = m[7], t5 = V.z, t4 = m[11];
  const float W = t1 * t0 + t3 * t2 + t5 * t4 + m[15];
  const float t8 = V.x, t3b = V.y, t12 = V.z;
  const float t7 = which_y ? m[1] : m[0];
  const float t9 = which_y ? m[5] : m[4];
  const float t11 = which_y ? m[9] : m[8];
  const float t13r = t8 * t7 + t3b * t9 + t12 * t11 + (which_y ? m[13] : m[12]);
  const float t13 = which_y ? -t13r : t13r;
  const float t6 = W;
  const float t14 = which_y ? cam[81] : cam[80];
  float d_xNDC = 0.0f, d_W = 0.0f;
  d[0] = d[1] = d[2] = 0.0f;
  {
    const float r14 = 1 * t14;
    const float r15 = r14 * 0.5f;
    d_xNDC += r15;
  }
  {
    const float r6 = d_xNDC / t6;
    const float s6 = which_y ? -r6 : r6;
    d[0] += s6 * t7;
    d[1] += s6 * t9;
    d[2] += s6 * t11;
    const float r13 = d_xNDC * -t13 / (t6 * t6);
    d_W += r13;
  }
  d[0] += d_W * t0;
  d[1] += d_W * t2;
  d[2] += d_W * t4;
}

static void edge_derivatives(const prep_t* s, const dmap_t* dm, int mode, const orc_model_params* mp, const float* cam,
                             const float* adj, int num_samples, const float* rnd, float* dscene, const float* tr_inv0) {
  const int W = (int)cam[80], H = (int)cam[81];
  /* (1) project every flattened vertex; z stays the world z (drender.h:258-267) */
  float* p2 = (float*)malloc(sizeof(float) * 3 * (s->total > 0 ? s->total : 1));
  for (int k = 0; k < s->total; k++) {
    float o[2];
    vertex_shader(cam, s->pos[k].x, s->pos[k].y, s->pos[k].z, o);
    p2[3 * k] = o[0]; p2[3 * k + 1] = o[1]; p2[3 * k + 2] = s->pos[k].z;
  }
  /* unique edges of the differentiable meshes, ordered by (v0, v1); the
   * first inserted wins on duplicates (std::set<Edge>, drender.h:244-299) */
  int ne_all = 0;
  for (int i = 0; i < s->n_meshes; i++)
    if (dm->by_mesh[i] >= 0) ne_all += 3 * (s->meshes[i].n_indices / 3) * s->meshes[i].n_instances;
  edge_t* E = (edge_t*)malloc(sizeof(edge_t) * (ne_all > 0 ? ne_all : 1));
  int ne = 0;
  int tri_base = 0; /* first traced triangle of the current (mesh, instance) block */
  for (int i = 0; i < s->n_meshes; i++) {
    const orc_mesh* m = s->meshes + i;
    if (dm->by_mesh[i] < 0) {
      tri_base += m->n_instances * (m->n_indices / 3);
      continue;
    }
    for (int j = 0; j < m->n_instances; j++, tri_base += m->n_indices / 3) {
      for (int k = 0; k + 2 < m->n_indices; k += 3) {
        int g[3] = {get_index(s, i, j, k), get_index(s, i, j, k + 1), get_index(s, i, j, k + 2)};
        int n[3] = {(int)m->indices[k], (int)m->indices[k + 1], (int)m->indices[k + 2]};
        for (int e = 0; e < 3; e++) {
          int a = e, b = (e + 1) % 3;
          edge_t ed;
          if (g[a] < g[b]) { ed.v0 = g[a]; ed.vn0 = n[a]; ed.v1 = g[b]; ed.vn1 = n[b]; }
          else { ed.v0 = g[b]; ed.vn0 = n[b]; ed.v1 = g[a]; ed.vn1 = n[a]; }
          ed.mesh = i;
          ed.inst = j;
          ed.tri0 = tri_base + k / 3;
          ed.tri1 = -1;
          E[ne++] = ed;
        }
      }
    }
  }
  /* stable ordering: sort by key, keep first occurrence (insertion order) */
  {
    /* tag with insertion index to make qsort stable */
    int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (ne > 0 ? ne : 1));
    edge_t* T = (edge_t*)malloc(sizeof(edge_t) * (ne > 0 ? ne : 1));
    for (int k = 0; k < ne; k++) order[k] = k;
    /* simple merge sort on (v0, v1, insertion index) */
    int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * (ne > 0 ? ne : 1));
    for (int width = 1; width < ne; width *= 2) {
      for (int lo = 0; lo < ne; lo += 2 * width) {
        int mid = lo + width < ne ? lo + width : ne;
        int hi = lo + 2 * width < ne ? lo + 2 * width : ne;
        int a = lo, b = mid, o = lo;
        while (a < mid && b < hi) {
          if (edge_cmp(&E[order[b]], &E[order[a]]) < 0) tmp[o++] = order[b++];
          else tmp[o++] = order[a++];
        }
        while (a < mid) tmp[o++] = order[a++];
        while (b < hi) tmp[o++] = order[b++];
      }
      memcpy(order, tmp, sizeof(int64_t) * ne);
    }
    int u = 0;
    for (int k = 0; k < ne; k++) {
      const edge_t* e = &E[order[k]];
      if (u > 0 && T[u - 1].v0 == e->v0 && T[u - 1].v1 == e->v1) {
        if (T[u - 1].tri1 < 0) T[u - 1].tri1 = e->tri0;
        continue;
      }
      T[u++] = *e;
    }
    memcpy(E, T, sizeof(edge_t) * u);
    ne = u;
    free(order); free(T); free(tmp);
  }
  if (ne == 0) { free(E); free(p2); return; }
  /* (2) build_edge_sampler: pmf by 3-D length of the projected points */
  float* pmf = (float*)malloc(sizeof(float) * ne);
  float* cdf = (float*)malloc(sizeof(float) * (ne + 1));
  cdf[0] = 0.0f;
  for (int k = 0; k < ne; k++) {
    const f3 a = v3(p2[3 * E[k].v0], p2[3 * E[k].v0 + 1], p2[3 * E[k].v0 + 2]);
    const f3 b = v3(p2[3 * E[k].v1], p2[3 * E[k].v1 + 1], p2[3 * E[k].v1 + 2]);
    pmf[k] = len3(sub3(b, a));
    if (mp->edge_set == 1 && E[k].tri1 >= 0) {
      /* silhouette edges only (no reference counterpart): both triangles
       * facing the eye, or both facing away, give the edge weight 0 */
      const f3 eye = v3(cam[64 + 12], cam[64 + 13], cam[64 + 14]); /* wv_inv * (0,0,0,1) */
      int facing[2];
      for (int q = 0; q < 2; q++) {
        const int t = q ? E[k].tri1 : E[k].tri0;
        const f3 A = s->pos[s->tri_gid[3 * t]], B = s->pos[s->tri_gid[3 * t + 1]], C = s->pos[s->tri_gid[3 * t + 2]];
        facing[q] = dot3(cross3(sub3(B, A), sub3(C, A)), sub3(A, eye)) < 0.0f;
      }
      if (facing[0] == facing[1]) pmf[k] = 0.0f;
    }
    cdf[k + 1] = pmf[k] + cdf[k];
  }
  const float length_sum = cdf[ne];
  for (int k = 0; k < ne; k++) pmf[k] /= length_sum;
  for (int k = 0; k <= ne; k++) cdf[k] /= length_sum;
  /* (3) samples, 14 static blocks with their own accumulators */
  ctx_t c = {s, cam, mode, mp};
  int64_t pos_total = 0, tr_total = 0;
  for (int k = 0; k < dm->n; k++) { pos_total += 3 * dm->lay[k].vertices; tr_total += 12 * dm->lay[k].instances; }
  float* dpos = (float*)calloc((size_t)REF_THREADS * (pos_total + 1), sizeof(float));
  float* dtr = (float*)calloc((size_t)REF_THREADS * (tr_total + 1), sizeof(float));
  int64_t pos_base[16], tr_base[16];
  {
    int64_t a = 0, b = 0;
    for (int k = 0; k < dm->n; k++) { pos_base[k] = a; tr_base[k] = b; a += 3 * dm->lay[k].vertices; b += 12 * dm->lay[k].instances; }
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
  for (int th = 0; th < REF_THREADS; th++) {
    int64_t b, e;
    static_block(num_samples, REF_THREADS, th, &b, &e);
    float* my_pos = dpos + (int64_t)th * (pos_total + 1);
    float* my_tr = dtr + (int64_t)th * (tr_total + 1);
    for (int64_t i = b; i < e; i++) {
      const float rnd0 = rnd[2 * i], rnd1 = rnd[2 * i + 1];
      /* sample(): clamp(upper_bound(cdf, u) - 1, 0, E-1) */
      int lo = 0, hi = ne + 1;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (rnd0 < cdf[mid]) hi = mid; else lo = mid + 1;
      }
      const int edge_id = clampi(lo - 1, 0, ne - 1);
      if (mp->edge_set == 1 && !(pmf[edge_id] > 0.0f)) continue; /* no silhouette edge in this view */
      const edge_t ed = E[edge_id];
      const float pm = pmf[edge_id];
      const f2 v0 = v2(p2[3 * ed.v0], p2[3 * ed.v0 + 1]);
      const f2 v1 = v2(p2[3 * ed.v1], p2[3 * ed.v1 + 1]);
      const float t = rnd1;
      const f2 p = add2(v0, scl2(sub2(v1, v0), t));
      const int xi = (int)p.x, yi = (int)p.y;
      if (xi < 0 || yi < 0 || xi >= W || yi >= H) continue;
      const float* av = adj + 3 * ((int64_t)yi * W + xi);
      const f3 a3 = v3(av[0], av[1], av[2]);
      if (len3(a3) < 1e-3f) continue;
      const f2 d = sub2(v1, v0);
      const float dl = len2(d);
      const f2 dn = v2(d.x / dl, d.y / dl);
      const f2 n = v2(-dn.y, dn.x); /* normal2D, utils.h:29 */
      const f2 cin = sub2(p, scl2(n, 1e-3f));
      const f2 cout = add2(p, scl2(n, 1e-3f));
      const uint32_t key_in = 0xA511E9B3u ^ (uint32_t)(i * 2u) * 2654435761u;
      const uint32_t key_out = 0xA511E9B3u ^ (uint32_t)(i * 2u + 1u) * 2654435761u;
      const f3 color_in = shade_sample(&c, cin, key_in);
      const f3 color_out = shade_sample(&c, cout, key_out);
      const float pdf = pm / len2(sub2(v1, v0));
      const float weight = 1.0f / (pdf * (float)num_samples);
      const float adjv = dot3(sub3(color_in, color_out), a3);
      if (!(adjv * adjv > 0.0f)) continue;
      /* d_v0 = float2{(1-t)*n.x, (1-t)*n.y} * adj * weight */
      const float d0x = (1 - t) * n.x * adjv * weight, d0y = (1 - t) * n.y * adjv * weight;
      const float d1x = t * n.x * adjv * weight, d1y = t * n.y * adjv * weight;
      /* edge_grad, drender.cpp:31-87 */
      const f3 v0_3d = s->pos[ed.v0], v1_3d = s->pos[ed.v1];
      float g0x[3], g0y[3], g1x[3], g1y[3];
      vs_grad(cam, v0_3d, 0, g0x);
      vs_grad(cam, v0_3d, 1, g0y);
      vs_grad(cam, v1_3d, 0, g1x);
      vs_grad(cam, v1_3d, 1, g1y);
      const int exact = mp->edge_jacobian != 0;
      float dv0_dx, dv0_dy, dv1_dx, dv1_dy;
      if (exact) {
        /* no reference counterpart: the full Jacobian of the endpoint's pixel
         * position, transposed (world-space gradient of each endpoint) */
        dv0_dx = g0x[0] * d0x + g0y[0] * d0y;
        dv0_dy = g0x[1] * d0x + g0y[1] * d0y;
        dv1_dx = g1x[0] * d1x + g1y[0] * d1y;
        dv1_dy = g1x[1] * d1x + g1y[1] * d1y;
      } else {
        dv0_dx = g0x[0] * d0x;
        dv0_dy = g0y[1] * d0y;
        dv1_dx = g1x[0] * d1x;
        dv1_dy = g1y[1] * d1y;
      }
      const float dv0_dz = (g0x[2] * d0x + g0y[2] * d0y);
      const float dv1_dz = (g1x[2] * d1x + g1y[2] * d1y);
      const int slot = dm->by_mesh[ed.mesh];
      const f3 v0o = s->orig[ed.v0], v1o = s->orig[ed.v1];
      float* P = my_pos + pos_base[slot];
      if (exact) {
        /* world = T * local: the transpose of the edge's own instance transform */
        const float* T = s->tr + 16 * (s->mesh_block0[ed.mesh] + ed.inst);
        P[ed.vn0 * 3 + 0] += M(T, 0, 0) * dv0_dx + M(T, 1, 0) * dv0_dy + M(T, 2, 0) * dv0_dz;
        P[ed.vn0 * 3 + 1] += M(T, 0, 1) * dv0_dx + M(T, 1, 1) * dv0_dy + M(T, 2, 1) * dv0_dz;
        P[ed.vn0 * 3 + 2] += M(T, 0, 2) * dv0_dx + M(T, 1, 2) * dv0_dy + M(T, 2, 2) * dv0_dz;
        P[ed.vn1 * 3 + 0] += M(T, 0, 0) * dv1_dx + M(T, 1, 0) * dv1_dy + M(T, 2, 0) * dv1_dz;
        P[ed.vn1 * 3 + 1] += M(T, 0, 1) * dv1_dx + M(T, 1, 1) * dv1_dy + M(T, 2, 1) * dv1_dz;
        P[ed.vn1 * 3 + 2] += M(T, 0, 2) * dv1_dx + M(T, 1, 2) * dv1_dy + M(T, 2, 2) * dv1_dz;
      } else {
        const float* tr = tr_inv0 + 16 * ed.inst; /* get_transform_inv(0)[inst] */
        P[ed.vn0 * 3 + 0] += M(tr, 0, 0) * dv0_dx + M(tr, 0, 1) * dv0_dy + M(tr, 0, 2) * dv0_dz;
        P[ed.vn0 * 3 + 1] += M(tr, 1, 0) * dv0_dx + M(tr, 1, 1) * dv0_dy + M(tr, 1, 2) * dv0_dz;
        P[ed.vn0 * 3 + 2] += M(tr, 2, 0) * dv0_dx + M(tr, 2, 1) * dv0_dy + M(tr, 2, 2) * dv0_dz;
        P[ed.vn1 * 3 + 0] += M(tr, 0, 0) * dv1_dx + M(tr, 0, 1) * dv1_dy + M(tr, 0, 2) * dv1_dz;
        P[ed.vn1 * 3 + 1] += M(tr, 1, 0) * dv1_dx + M(tr, 1, 1) * dv1_dy + M(tr, 1, 2) * dv1_dz;
        P[ed.vn1 * 3 + 2] += M(tr, 2, 0) * dv1_dx + M(tr, 2, 1) * dv1_dy + M(tr, 2, 2) * dv1_dz;
      }
      float* T = my_tr + tr_base[slot] + 12 * ed.inst;
      T[0] += v0o.x * dv0_dx + v1o.x * dv1_dx;
      T[1] += v0o.y * dv0_dx + v1o.y * dv1_dx;
      T[2] += v0o.z * dv0_dx + v1o.z * dv1_dx;
      T[3] += 1 * dv0_dx + 1 * dv1_dx;
      T[4] += v0o.x * dv0_dy + v1o.x * dv1_dy;
      T[5] += v0o.y * dv0_dy + v1o.y * dv1_dy;
      T[6] += v0o.z * dv0_dy + v1o.z * dv1_dy;
      T[7] += 1 * dv0_dy + 1 * dv1_dy;
      T[8] += v0o.x * dv0_dz + v1o.x * dv1_dz;
      T[9] += v0o.y * dv0_dz + v1o.y * dv1_dz;
      T[10] += v0o.z * dv0_dz + v1o.z * dv1_dz;
      T[11] += 1 * dv0_dz + 1 * dv1_dz;
    }
  }
  /* reduction in thread order (drender.h:380-397) */
  for (int k = 0; k < dm->n; k++) {
    float* g = dscene + dm->base[k];
    const dlayout_t* L = dm->lay + k;
    for (int th = 0; th < REF_THREADS; th++) {
      const float* P = dpos + (int64_t)th * (pos_total + 1) + pos_base[k];
      for (int j = 0; j < 3 * L->vertices; j++) g[L->pos_off + j] += P[j];
    }
    if (L->tr_off >= 0) {
      for (int th = 0; th < REF_THREADS; th++) {
        const float* T = dtr + (int64_t)th * (tr_total + 1) + tr_base[k];
        for (int j = 0; j < 12 * L->instances; j++) g[L->tr_off + j] += T[j];
      }
    } else {
      /* restricted: the matrix gradient through the Jacobian of to_mat (drender.h:398-421) */
      float* mat = (float*)calloc(12 * (size_t)L->instances, sizeof(float));
      for (int th = 0; th < REF_THREADS; th++) {
        const float* T = dtr + (int64_t)th * (tr_total + 1) + tr_base[k];
        for (int j = 0; j < 12 * L->instances; j++) mat[j] += T[j];
      }
      const float* rp = s->meshes[dm->ids[k]].restricted;
      for (int j = 0; j < L->instances; j++) {
        float jac[84];
        orc_restricted_jacobian(rp + 7 * j, jac);
        for (int q = 0; q < 7; q++)
          for (int l = 0; l < 12; l++) g[L->rt_off + 7 * j + q] += jac[12 * q + l] * mat[12 * j + l];
      }
      free(mat);
    }
  }
  free(dpos); free(dtr); free(pmf); free(cdf); free(E); free(p2);
}

void orc_prng(int seed, int count, float* out) {
  /* prng::RandomGenInit / NextState / rndFloat, qmc.h:81-87, qmc.cpp:250-268 */
  /* the reference computes these in int and relies on two's-complement
   * wrap-around; unsigned arithmetic yields the same bits without overflow */
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

void orc_edge_random_table(int num_samples, int num_threads, float* out) {
  for (int k = 0; k < num_threads; k++) {
    int64_t b, e;
    static_block(num_samples, num_threads, k, &b, &e);
    if (e <= b) continue;
    orc_prng(7777 + k * k + 1, (int)(2 * (e - b)), out + 2 * b);
  }
}

void orc_hammersley(int n, float* out) {
  /* qmc::planeHammersley, qmc.cpp:227-243 */
  for (int k = 0; k < n; k++) {
    float u = 0;
    int kk = k;
    for (float p = 0.5f; kk; p *= 0.5f, kk >>= 1)
      if (kk & 1) u += p;
    float v = (k + 0.5f) / n;
    out[2 * k + 0] = u;
    out[2 * k + 1] = v;
  }
}

/* d_render over views: interior then edges per view (drender.h:154-166). */
static int d_render_prepared(const prep_t* s, const dmap_t* dm, int mode, int spp, const orc_model_params* mp,
                             const float* cams, int n_views, const float* adjoints, int edge_samples, float* dscene,
                             const float* tr_inv0) {
  float* rnd = (float*)malloc(sizeof(float) * 2 * (edge_samples > 0 ? edge_samples : 1));
  orc_edge_random_table(edge_samples, REF_THREADS, rnd);
  int64_t off = 0;
  for (int vi = 0; vi < n_views; vi++) {
    const float* cam = cams + ORC_CAM_FLOATS * vi;
    const float* adj = adjoints + off;
    if (mode != ORC_SILHOUETTE) interior_derivatives(s, dm, mode, spp, mp, cam, adj, dscene, (uint32_t)vi * 0x9E3779B9u);
    edge_derivatives(s, dm, mode, mp, cam, adj, edge_samples, rnd, dscene, tr_inv0);
    off += 3 * (int64_t)cam[80] * (int64_t)cam[81];
  }
  free(rnd);
  return 0;
}

int orc_d_render(const orc_mesh* meshes, int n_meshes, int mode, int spp, const orc_model_params* mp, const float* cams,
                 int n_views, const float* adjoints, int edge_samples, const int32_t* ids, int n_ids, float* dscene) {
  orc_model_params dmp;
  if (!mp) { orc_default_model_params(&dmp); mp = &dmp; }
  dmap_t dm;
  if (dmap_build(&dm, meshes, n_meshes, mode, ids, n_ids) != 0) return -1;
  prep_t s;
  prep_build(&s, meshes, n_meshes);
  int r = d_render_prepared(&s, &dm, mode, spp, mp, cams, n_views, adjoints, edge_samples, dscene, s.tr_inv);
  prep_free(&s);
  return r;
}

/* LossAndDiffLoss, utils.cpp:15-27 */
static float loss_and_diff(const float* b, const float* a, float* out, int64_t n) {
  double acc = 0.0;
  for (int64_t i = 0; i < n; i++) {
    const f3 d = v3(b[3 * i] - a[3 * i], b[3 * i + 1] - a[3 * i + 1], b[3 * i + 2] - a[3 * i + 2]);
    out[3 * i] = 2.0f * d.x; out[3 * i + 1] = 2.0f * d.y; out[3 * i + 2] = 2.0f * d.z;
    acc += (double)dot3(d, d);
  }
  return (float)acc;
}

static int d_render_and_compare_prepared(const prep_t* s, const dmap_t* dm, int mode, int spp,
                                         const orc_model_params* mp, const float* cams, int n_views,
                                         const float* targets, int edge_samples, float* dscene, float* out_images,
                                         float* loss, const float* tr_inv0) {
  int64_t tot = 0;
  for (int vi = 0; vi < n_views; vi++) tot += 3 * (int64_t)cams[ORC_CAM_FLOATS * vi + 80] * (int64_t)cams[ORC_CAM_FLOATS * vi + 81];
  float* imgs = out_images ? out_images : (float*)malloc(sizeof(float) * tot);
  float* adj = (float*)malloc(sizeof(float) * tot);
  int64_t off = 0;
  for (int vi = 0; vi < n_views; vi++) {
    const float* cam = cams + ORC_CAM_FLOATS * vi;
    render_view(s, mode, spp, mp, cam, imgs + off, (uint32_t)vi * 0x9E3779B9u);
    off += 3 * (int64_t)cam[80] * (int64_t)cam[81];
  }
  /* adjoints sized like view 0 (drender.h:180-182) */
  const int64_t n0 = (int64_t)cams[80] * (int64_t)cams[81];
  float mse = 0.0f;
  off = 0;
  for (int vi = 0; vi < n_views; vi++) {
    mse += loss_and_diff(imgs + off, targets + off, adj + 3 * n0 * vi, n0);
    off += 3 * (int64_t)cams[ORC_CAM_FLOATS * vi + 80] * (int64_t)cams[ORC_CAM_FLOATS * vi + 81];
  }
  memset(dscene, 0, sizeof(float) * dm->total);
  d_render_prepared(s, dm, mode, spp, mp, cams, n_views, adj, edge_samples, dscene, tr_inv0);
  if (loss) *loss = mse / (float)(n_views * (int)cams[80] * (int)cams[81]);
  free(adj);
  if (!out_images) free(imgs);
  return 0;
}

int orc_d_render_and_compare(const orc_mesh* meshes, int n_meshes, int mode, int spp, const orc_model_params* mp,
                             const float* cams, int n_views, const float* targets, int edge_samples,
                             const int32_t* ids, int n_ids, float* dscene, float* out_images, float* loss) {
  orc_model_params dmp;
  if (!mp) { orc_default_model_params(&dmp); mp = &dmp; }
  dmap_t dm;
  if (dmap_build(&dm, meshes, n_meshes, mode, ids, n_ids) != 0) return -1;
  prep_t s;
  prep_build(&s, meshes, n_meshes);
  int r = d_render_and_compare_prepared(&s, &dm, mode, spp, mp, cams, n_views, targets, edge_samples, dscene,
                                        out_images, loss, s.tr_inv);
  prep_free(&s);
  return r;
}

/* ---------------------------------------------------------------------------
 * Optimiser (optimizer.h:9-50, optimizer_simple.cpp:13-309).
 * ------------------------------------------------------------------------- */
void orc_opt_params_default(int alg, orc_opt_params* p) {
  memset(p, 0, sizeof(*p));
  p->alg = alg;
  p->decay_period = 25;
  p->decay_mult = 0.75f;
  p->base_lr = 0.1f;
  p->position_lr = 0.1f;
  p->textures_lr = 0.1f;
  p->transforms_lr = 0.1f;
  p->flags = 1 | 2 | 4 | 8;
  p->n_dmesh_ids = 1;
  p->dmesh_ids[0] = 0;
  if (alg == 4) p->decay_period = 100; /* set_default, optimizer_simple.cpp:13-23 */
}

int orc_optimize(const orc_mesh* meshes_in, int n_meshes, int mode, int spp, const orc_model_params* mp,
                 const float* cams, int n_views, const float* targets, const orc_opt_params* P, int iters,
                 float* final_error, float* losses, float* traj_v, float* traj_c, float* traj_t, float* traj_tr,
                 float* traj_rt) {
  orc_model_params dmp;
  if (!mp) { orc_default_model_params(&dmp); mp = &dmp; }
  /* private copy of the scene (OptSimple::m_scene) */
  orc_mesh* ms = (orc_mesh*)malloc(sizeof(orc_mesh) * n_meshes);
  float** vbuf = (float**)calloc(n_meshes, sizeof(float*));
  float** cbuf = (float**)calloc(n_meshes, sizeof(float*));
  float** tbuf = (float**)calloc(n_meshes, sizeof(float*));
  float** trbuf = (float**)calloc(n_meshes, sizeof(float*));
  float** rbuf = (float**)calloc(n_meshes, sizeof(float*));
  for (int i = 0; i < n_meshes; i++) {
    ms[i] = meshes_in[i];
    vbuf[i] = (float*)malloc(sizeof(float) * 3 * ms[i].n_vertices);
    memcpy(vbuf[i], meshes_in[i].vertices, sizeof(float) * 3 * ms[i].n_vertices);
    ms[i].vertices = vbuf[i];
    if (ms[i].colors) {
      cbuf[i] = (float*)malloc(sizeof(float) * 3 * ms[i].n_vertices);
      memcpy(cbuf[i], meshes_in[i].colors, sizeof(float) * 3 * ms[i].n_vertices);
      ms[i].colors = cbuf[i];
    }
    if (ms[i].texture) {
      size_t nt = (size_t)ms[i].tex_w * ms[i].tex_h * ms[i].tex_channels;
      tbuf[i] = (float*)malloc(sizeof(float) * nt);
      memcpy(tbuf[i], meshes_in[i].texture, sizeof(float) * nt);
      ms[i].texture = tbuf[i];
    }
    if (meshes_in[i].restricted) {
      rbuf[i] = (float*)malloc(sizeof(float) * 7 * ms[i].n_instances);
      memcpy(rbuf[i], meshes_in[i].restricted, sizeof(float) * 7 * ms[i].n_instances);
      ms[i].restricted = rbuf[i];
    }
    trbuf[i] = (float*)malloc(sizeof(float) * 16 * ms[i].n_instances);
    for (int j = 0; j < ms[i].n_instances; j++) {
      float tmp[16];
      memcpy(trbuf[i] + 16 * j, mesh_tr(ms + i, j, tmp), 16 * sizeof(float));
    }
    ms[i].transforms = trbuf[i];
  }
  dmap_t dm;
  if (dmap_build(&dm, ms, n_meshes, mode, P->dmesh_ids, P->n_dmesh_ids) != 0) return -1;
  float* grad = (float*)calloc(dm.total, sizeof(float));
  float* G = (float*)calloc(dm.total, sizeof(float));
  float* mv = (float*)calloc(dm.total, sizeof(float));
  /* GetLR: {offset, lr} segments per DMesh (optimizer_simple.cpp:61-80) */
  float lr_val[16][4];
  int lr_off[16][4], lr_n[16];
  for (int k = 0; k < dm.n; k++) {
    int n = 0;
    lr_off[k][n] = 0; lr_val[k][n++] = P->position_lr;
    if (dm.lay[k].color_off >= 0) { lr_off[k][n] = dm.lay[k].color_off; lr_val[k][n++] = P->base_lr; }
    if (dm.lay[k].tex_off >= 0) { lr_off[k][n] = dm.lay[k].tex_off; lr_val[k][n++] = P->textures_lr; }
    lr_off[k][n] = dm.lay[k].tr_off >= 0 ? dm.lay[k].tr_off : dm.lay[k].rt_off; lr_val[k][n++] = P->transforms_lr;
    lr_n[k] = n;
  }
  /* the inverse of mesh 0's transforms is taken once, at the first prepare
   * (Scene::prepare_for_render appends to transforms_inv, scene_utils.cpp:118-129) */
  float* tr_inv0 = (float*)malloc(sizeof(float) * 16 * ms[0].n_instances);
  for (int j = 0; j < ms[0].n_instances; j++) mat_inverse(ms[0].transforms + 16 * j, tr_inv0 + 16 * j);
  int64_t off_v = 0, off_c = 0, off_t = 0, off_tr = 0, off_rt = 0;
  float err = 0.0f;
  for (int it = 0; it < iters; it++) {
    prep_t s;
    prep_build(&s, ms, n_meshes);
    d_render_and_compare_prepared(&s, &dm, mode, spp, mp, cams, n_views, targets,
                                  (int)cams[80] * (int)cams[81], grad, NULL, &err, tr_inv0);
    prep_free(&s);
    if (losses) losses[it] = err;
    /* OptStep, optimizer_simple.cpp:188-236 */
    int64_t off = 0;
    for (int k = 0; k < dm.n; k++) {
      float* g = grad + dm.base[k];
      const int full = dm.lay[k].full;
      if (P->alg >= 2) {
        if (P->alg == 2) {
          for (int i = 0; i < full; i++) G[off + i] += (g[i] * g[i]);
        } else if (P->alg == 3) {
          const float alpha = 0.5f;
          for (int i = 0; i < full; i++) G[off + i] = 2.0f * (G[off + i] * alpha + (g[i] * g[i]) * (1.0f - alpha));
        } else if (P->alg == 4) {
          const float alpha = 0.5f, beta = 0.25f;
          for (int i = 0; i < full; i++) mv[off + i] = mv[off + i] * beta + g[i] * (1.0f - beta);
          for (int i = 0; i < full; i++) G[off + i] = 2.0f * (G[off + i] * alpha + (g[i] * g[i]) * (1.0f - alpha));
          for (int i = 0; i < full; i++) g[i] = mv[off + i];
        }
        /* reads G[i], not G[off+i] (optimizer_simple.cpp:224) */
        for (int i = 0; i < full; i++) g[i] = g[i] / (sqrtf(G[i] + 1e-8f));
      }
      for (int q = 0; q < lr_n[k]; q++) {
        int next = (q == lr_n[k] - 1) ? full : lr_off[k][q + 1];
        for (int j = lr_off[k][q]; j < next; j++) g[j] *= lr_val[k][q];
      }
      off += full;
    }
    /* OptUpdateScene, optimizer_simple.cpp:92-186 */
    for (int k = 0; k < dm.n; k++) {
      const int mid = dm.ids[k];
      orc_mesh* m = ms + mid;
      const float* g = grad + dm.base[k];
      const dlayout_t* L = dm.lay + k;
      if (P->flags & 1)
        for (int v = 0; v < 3 * m->n_vertices; v++) vbuf[mid][v] -= g[L->pos_off + v];
      if ((P->flags & 2) && L->tr_off >= 0)
        for (int j = 0; j < m->n_instances; j++)
          for (int r = 0; r < 3; r++)
            for (int c2 = 0; c2 < 4; c2++) M(trbuf[mid] + 16 * j, r, c2) -= g[L->tr_off + 12 * j + 4 * r + c2];
      if ((P->flags & 2) && L->rt_off >= 0) {
        /* translate, rotate, scale -= step; the matrices follow at the next prepare */
        for (int j = 0; j < 7 * m->n_instances; j++) rbuf[mid][j] -= g[L->rt_off + j];
        for (int j = 0; j < m->n_instances; j++) orc_restricted_to_mat(rbuf[mid] + 7 * j, trbuf[mid] + 16 * j);
      }
      if (L->color_off >= 0 && (P->flags & 4) && cbuf[mid])
        for (int v = 0; v < 3 * m->n_vertices; v++) cbuf[mid][v] -= g[L->color_off + v];
      if (mode != ORC_SILHOUETTE && mode != ORC_VERTEX_COLOR && (P->flags & 8) && L->tex_off >= 0 && tbuf[mid]) {
        size_t nt = (size_t)m->tex_w * m->tex_h * m->tex_channels;
        for (size_t j = 0; j < nt; j++) tbuf[mid][j] -= g[L->tex_off + j];
      }
    }
    /* StepDecay, optimizer_simple.cpp:82-90 */
    if (it > 0 && it % P->decay_period == 0)
      for (int k = 0; k < dm.n; k++)
        for (int q = 0; q < lr_n[k]; q++) lr_val[k][q] *= P->decay_mult;
    /* trajectory */
    for (int i = 0; i < n_meshes; i++) {
      if (traj_v) { memcpy(traj_v + off_v, vbuf[i], sizeof(float) * 3 * ms[i].n_vertices); off_v += 3 * ms[i].n_vertices; }
      if (traj_c && cbuf[i]) { memcpy(traj_c + off_c, cbuf[i], sizeof(float) * 3 * ms[i].n_vertices); off_c += 3 * ms[i].n_vertices; }
      if (traj_t && tbuf[i]) {
        size_t nt = (size_t)ms[i].tex_w * ms[i].tex_h * ms[i].tex_channels;
        memcpy(traj_t + off_t, tbuf[i], sizeof(float) * nt);
        off_t += nt;
      }
      if (traj_tr) { memcpy(traj_tr + off_tr, trbuf[i], sizeof(float) * 16 * ms[i].n_instances); off_tr += 16 * ms[i].n_instances; }
      if (traj_rt && rbuf[i]) { memcpy(traj_rt + off_rt, rbuf[i], sizeof(float) * 7 * ms[i].n_instances); off_rt += 7 * ms[i].n_instances; }
    }
  }
  if (final_error) *final_error = err;
  for (int i = 0; i < n_meshes; i++) { free(vbuf[i]); free(cbuf[i]); free(tbuf[i]); free(trbuf[i]); free(rbuf[i]); }
  free(vbuf); free(cbuf); free(tbuf); free(trbuf); free(rbuf); free(ms);
  free(grad); free(G); free(mv); free(tr_inv0);
  return 0;
}
