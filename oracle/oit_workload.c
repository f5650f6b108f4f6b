/* The synthetic workload of the oracle's CPU legs: seeded sphere scenes and
 * the camera, restated from the engine's own generator (scene.cpp, the
 * oit_scene_generate / oit_camera entry points) so that a process timing the
 * oracle loads no product code. TEST INFRASTRUCTURE: tests/test_oracle_workload.py
 * checks every output against the engine's generator bit for bit.
 *
 * The reference builds its scene with std::default_random_engine(3625)
 * (main.cpp:350), an implementation-defined sequence, and
 * nvutils::createSphereUv (main.cpp:346); both sides here use the engine's
 * SplitMix64 stream and UV sphere instead. Double-precision trigonometry from
 * the host's libm, -ffp-contract=off: the same bits as the engine on the same
 * host. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include "oit_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static uint64_t splitmix_next(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static float splitmix_uniform(uint64_t* s) { return (float)(splitmix_next(s) >> 40) * (1.0f / 16777216.0f); }

static int desc_ok(uint32_t num_objects, uint32_t stacks, uint32_t slices, float rmin, float rmax) {
  return num_objects > 0 && stacks >= 2 && slices >= 3 && stacks <= 1024 && slices <= 1024 && rmin >= 0.0f &&
         rmax >= rmin;
}

int or_scene_size(uint32_t num_objects, uint32_t stacks, uint32_t slices, uint32_t* num_vertices,
                  uint32_t* num_triangles, uint32_t* triangles_per_object) {
  if (!desc_ok(num_objects, stacks, slices, 0.0f, 0.0f)) return -1;
  const uint64_t vpo = (uint64_t)(stacks + 1) * (slices + 1), tpo = (uint64_t)slices * (2 * (stacks - 2) + 2);
  if (vpo * num_objects > 0xFFFFFFFFull || tpo * num_objects > 0xFFFFFFFFull / 3) return -1;
  if (num_vertices) *num_vertices = (uint32_t)(vpo * num_objects);
  if (num_triangles) *num_triangles = (uint32_t)(tpo * num_objects);
  if (triangles_per_object) *triangles_per_object = (uint32_t)tpo;
  return 0;
}

/* One outward-wound triangle of the unit sphere template: (b - a) x (c - a)
 * points away from the centre, else b and c swap. */
static void emit_tri(const float* tp, uint32_t* tt, uint32_t* k, uint32_t a, uint32_t b, uint32_t c) {
  const float* A = tp + 3 * (size_t)a;
  const float* B = tp + 3 * (size_t)b;
  const float* C = tp + 3 * (size_t)c;
  const double ux = B[0] - A[0], uy = B[1] - A[1], uz = B[2] - A[2];
  const double vx = C[0] - A[0], vy = C[1] - A[1], vz = C[2] - A[2];
  const double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
  const double dd = nx * (A[0] + B[0] + C[0]) + ny * (A[1] + B[1] + C[1]) + nz * (A[2] + B[2] + C[2]);
  tt[3 * *k + 0] = a;
  tt[3 * *k + 1] = dd >= 0 ? b : c;
  tt[3 * *k + 2] = dd >= 0 ? c : b;
  ++*k;
}

int or_scene_generate(uint64_t seed, uint32_t num_objects, uint32_t stacks, uint32_t slices, float half_extent,
                      float radius_min, float radius_max, float* vertices, uint32_t* indices) {
  uint32_t nv, nt, tpo;
  if (!desc_ok(num_objects, stacks, slices, radius_min, radius_max) || !vertices || !indices ||
      or_scene_size(num_objects, stacks, slices, &nv, &nt, &tpo) != 0)
    return -1;
  const uint32_t vpo = (stacks + 1) * (slices + 1);
  float* tp = (float*)malloc(sizeof(float) * 3 * (size_t)vpo);
  uint32_t* tt = (uint32_t*)malloc(sizeof(uint32_t) * 3 * (size_t)tpo);
  if (!tp || !tt) {
    free(tp);
    free(tt);
    return -1;
  }
  for (uint32_t i = 0; i <= stacks; ++i) {
    const double th = M_PI * (double)i / (double)stacks;
    for (uint32_t j = 0; j <= slices; ++j) {
      const double ph = 2.0 * M_PI * (double)j / (double)slices;
      float* p = tp + 3 * (size_t)(i * (slices + 1) + j);
      p[0] = (float)(sin(th) * cos(ph));
      p[1] = (float)cos(th);
      p[2] = (float)(sin(th) * sin(ph));
    }
  }
  uint32_t k = 0;
  for (uint32_t i = 0; i < stacks; ++i)
    for (uint32_t j = 0; j < slices; ++j) {
      const uint32_t v00 = i * (slices + 1) + j, v01 = v00 + 1, v10 = v00 + (slices + 1), v11 = v10 + 1;
      if (i != 0) emit_tri(tp, tt, &k, v00, v10, v01);
      if (i != stacks - 1) emit_tri(tp, tt, &k, v01, v10, v11);
    }
  /* per object, in stream order: centre, radius, colour */
  uint64_t rng = seed;
  for (uint32_t o = 0; o < num_objects; ++o) {
    float q[8];
    q[0] = (splitmix_uniform(&rng) * 2.0f - 1.0f) * half_extent;
    q[1] = (splitmix_uniform(&rng) * 2.0f - 1.0f) * half_extent;
    q[2] = (splitmix_uniform(&rng) * 2.0f - 1.0f) * half_extent;
    q[3] = radius_min + splitmix_uniform(&rng) * (radius_max - radius_min);
    for (int c = 0; c < 4; ++c) q[4 + c] = splitmix_uniform(&rng);
    float* vo = vertices + 10 * (size_t)o * vpo;
    for (uint32_t v = 0; v < vpo; ++v) {
      const float* p = tp + 3 * (size_t)v;
      float* out = vo + 10 * (size_t)v;
      out[0] = p[0] * q[3] + q[0];
      out[1] = p[1] * q[3] + q[1];
      out[2] = p[2] * q[3] + q[2];
      out[3] = p[0];
      out[4] = p[1];
      out[5] = p[2];
      for (int c = 0; c < 4; ++c) out[6 + c] = q[4 + c];
    }
    uint32_t* io = indices + 3 * (size_t)o * tpo;
    for (uint32_t t = 0; t < 3 * tpo; ++t) io[t] = tt[t] + o * vpo;
  }
  free(tp);
  free(tt);
  return 0;
}

/* lookAt (right-handed, +y up) and a Vulkan perspective (depth in [0, 1],
 * y down), in double, rounded to float; column-major like SceneData. */
int or_camera(uint32_t width, uint32_t height, const float eye[3], const float target[3], float fov_y_degrees,
              float z_near, float z_far, float* proj_view16, float* view16) {
  if (!proj_view16 || !view16 || !eye || !target || !width || !height || !(z_near > 0.0f) || !(z_far > z_near) ||
      !(fov_y_degrees > 0.0f && fov_y_degrees < 180.0f))
    return -1;
  double f[3] = {(double)target[0] - eye[0], (double)target[1] - eye[1], (double)target[2] - eye[2]};
  const double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  if (!(fl > 0.0)) return -1;
  for (int i = 0; i < 3; ++i) f[i] /= fl;
  const double up[3] = {0.0, 1.0, 0.0};
  double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
  const double sl = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  if (!(sl > 0.0)) return -1;
  for (int i = 0; i < 3; ++i) s[i] /= sl;
  const double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
  const double V[4][4] = {{s[0], s[1], s[2], -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2])},
                          {u[0], u[1], u[2], -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2])},
                          {-f[0], -f[1], -f[2], (f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2])},
                          {0, 0, 0, 1}};
  const double t = 1.0 / tan(0.5 * (double)fov_y_degrees * M_PI / 180.0);
  const double aspect = (double)width / (double)height;
  const double n = z_near, fr = z_far;
  const double P[4][4] = {
      {t / aspect, 0, 0, 0}, {0, -t, 0, 0}, {0, 0, fr / (n - fr), n * fr / (n - fr)}, {0, 0, -1, 0}};
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 4; ++k) acc += P[r][k] * V[k][c];
      proj_view16[c * 4 + r] = (float)acc;
      view16[c * 4 + r] = (float)V[r][c];
    }
  return 0;
}
