// Host-side helpers of the C ABI that need no GPU: seeded sphere scenes, the
// camera, A-buffer sizing and the sRGB tables. Compiled with
// -ffp-contract=off so that x86-64 and aarch64 hosts generate bit-identical
// meshes.
#include <cmath>
#include <cstring>

#include "../../include/oit_gb300.h"
#include "oit_internal.h"

namespace {

// SplitMix64: the scene generator's own seeded stream (the reference uses
// std::default_random_engine(3625), main.cpp:350, whose sequence is
// implementation-defined).
struct SplitMix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
};

bool valid_desc(const oit_scene_desc* d) {
  return d && d->num_objects > 0 && d->stacks >= 2 && d->slices >= 3 && d->stacks <= 1024 && d->slices <= 1024 &&
         d->radius_min >= 0.0f && d->radius_max >= d->radius_min;
}

uint32_t sphere_vertices(const oit_scene_desc* d) { return (d->stacks + 1) * (d->slices + 1); }
uint32_t sphere_triangles(const oit_scene_desc* d) { return d->slices * (2 * (d->stacks - 2) + 2); }

// UV sphere (the role of nvutils::createSphereUv(1, 2*subdiv, subdiv),
// main.cpp:346): unit-radius positions (which are also the normals) and
// triangles wound counter-clockwise seen from outside.
void sphere_template(const oit_scene_desc* d, float* tp, uint32_t* tt) {
  const uint32_t stacks = d->stacks, slices = d->slices;
  for (uint32_t i = 0; i <= stacks; ++i) {
    const double th = M_PI * (double)i / (double)stacks;
    for (uint32_t j = 0; j <= slices; ++j) {
      const double ph = 2.0 * M_PI * (double)j / (double)slices;
      float* p = tp + 3 * (size_t)(i * (slices + 1) + j);
      p[0] = (float)(std::sin(th) * std::cos(ph));
      p[1] = (float)std::cos(th);
      p[2] = (float)(std::sin(th) * std::sin(ph));
    }
  }
  uint32_t k = 0;
  auto emit = [&](uint32_t a, uint32_t b, uint32_t c) {
    // orient outward: (b - a) x (c - a) must point away from the centre
    const float* A = tp + 3 * (size_t)a;
    const float* B = tp + 3 * (size_t)b;
    const float* C = tp + 3 * (size_t)c;
    const double ux = B[0] - A[0], uy = B[1] - A[1], uz = B[2] - A[2];
    const double vx = C[0] - A[0], vy = C[1] - A[1], vz = C[2] - A[2];
    const double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    const double dd = nx * (A[0] + B[0] + C[0]) + ny * (A[1] + B[1] + C[1]) + nz * (A[2] + B[2] + C[2]);
    tt[3 * k + 0] = a;
    tt[3 * k + 1] = dd >= 0 ? b : c;
    tt[3 * k + 2] = dd >= 0 ? c : b;
    ++k;
  };
  for (uint32_t i = 0; i < stacks; ++i) {
    for (uint32_t j = 0; j < slices; ++j) {
      const uint32_t v00 = i * (slices + 1) + j, v01 = v00 + 1;
      const uint32_t v10 = v00 + (slices + 1), v11 = v10 + 1;
      if (i != 0) emit(v00, v10, v01);
      if (i != stacks - 1) emit(v01, v10, v11);
    }
  }
}

// Per object, in stream order: centre, radius, colour (main.cpp:353-369 draws
// the same quantities). inst = centre.xyz, radius, color.rgba.
void instance_params(const oit_scene_desc* d, float* inst) {
  SplitMix64 rng{d->seed};
  for (uint32_t o = 0; o < d->num_objects; ++o) {
    float* q = inst + 8 * (size_t)o;
    q[0] = (rng.uniform() * 2.0f - 1.0f) * d->half_extent;
    q[1] = (rng.uniform() * 2.0f - 1.0f) * d->half_extent;
    q[2] = (rng.uniform() * 2.0f - 1.0f) * d->half_extent;
    q[3] = d->radius_min + rng.uniform() * (d->radius_max - d->radius_min);
    for (int c = 0; c < 4; ++c) q[4 + c] = rng.uniform();
  }
}

}  // namespace

extern "C" {

int oit_scene_size(const oit_scene_desc* desc, uint32_t* num_vertices, uint32_t* num_triangles,
                   uint32_t* triangles_per_object) {
  if (!valid_desc(desc)) return OIT_ERR_INVALID_ARGUMENT;
  const uint64_t v = (uint64_t)sphere_vertices(desc) * desc->num_objects;
  const uint64_t t = (uint64_t)sphere_triangles(desc) * desc->num_objects;
  if (v > 0xFFFFFFFFull || t > 0xFFFFFFFFull / 3) return OIT_ERR_INVALID_ARGUMENT;
  if (num_vertices) *num_vertices = (uint32_t)v;
  if (num_triangles) *num_triangles = (uint32_t)t;
  if (triangles_per_object) *triangles_per_object = sphere_triangles(desc);
  return OIT_OK;
}

// num_objects scaled and translated copies of the template flattened into one
// mesh (main.cpp:353-387): position = template * radius + centre, normal =
// template, colour = the object's.
int oit_scene_generate(const oit_scene_desc* desc, float* vertices, uint32_t* indices) {
  if (!valid_desc(desc) || !vertices || !indices) return OIT_ERR_INVALID_ARGUMENT;
  uint32_t nv = 0, nt = 0, tpo = 0;
  int st = oit_scene_size(desc, &nv, &nt, &tpo);
  if (st != OIT_OK) return st;
  const uint32_t vpo = sphere_vertices(desc);
  float* tp = new float[3 * (size_t)vpo];
  uint32_t* tt = new uint32_t[3 * (size_t)tpo];
  float* inst = new float[8 * (size_t)desc->num_objects];
  sphere_template(desc, tp, tt);
  instance_params(desc, inst);
  for (uint32_t o = 0; o < desc->num_objects; ++o) {
    const float* q = inst + 8 * (size_t)o;
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
    const uint32_t base = o * vpo;
    for (uint32_t t = 0; t < 3 * tpo; ++t) io[t] = tt[t] + base;
  }
  delete[] tp;
  delete[] tt;
  delete[] inst;
  return OIT_OK;
}

int oit_scene_generate_instanced(const oit_scene_desc* desc, float* template_vertices, uint32_t* template_indices,
                                 float* instances) {
  if (!valid_desc(desc) || !template_vertices || !template_indices || !instances) return OIT_ERR_INVALID_ARGUMENT;
  int st = oit_scene_size(desc, nullptr, nullptr, nullptr);
  if (st != OIT_OK) return st;
  const uint32_t vpo = sphere_vertices(desc);
  float* tp = new float[3 * (size_t)vpo];
  sphere_template(desc, tp, template_indices);
  for (uint32_t v = 0; v < vpo; ++v)
    for (int c = 0; c < 3; ++c) {
      template_vertices[6 * (size_t)v + c] = tp[3 * (size_t)v + c];
      template_vertices[6 * (size_t)v + 3 + c] = tp[3 * (size_t)v + c];
    }
  instance_params(desc, instances);
  delete[] tp;
  return OIT_OK;
}

// lookAt (right-handed, +y up) and a Vulkan perspective (depth in [0,1], y
// down), computed in double and rounded to float.
int oit_camera(uint32_t width, uint32_t height, const float eye[3], const float target[3], float fov_y_degrees,
               float z_near, float z_far, oit_scene_data* out) {
  if (!out || !eye || !target || !width || !height || !(z_near > 0.0f) || !(z_far > z_near) ||
      !(fov_y_degrees > 0.0f && fov_y_degrees < 180.0f))
    return OIT_ERR_INVALID_ARGUMENT;
  double f[3] = {(double)target[0] - eye[0], (double)target[1] - eye[1], (double)target[2] - eye[2]};
  double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  if (!(fl > 0.0)) return OIT_ERR_INVALID_ARGUMENT;
  for (double& x : f) x /= fl;
  const double up[3] = {0.0, 1.0, 0.0};
  double s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
  const double sl = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  if (!(sl > 0.0)) return OIT_ERR_INVALID_ARGUMENT;
  for (double& x : s) x /= sl;
  const double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
  double V[4][4] = {{s[0], s[1], s[2], -(s[0] * eye[0] + s[1] * eye[1] + s[2] * eye[2])},
                    {u[0], u[1], u[2], -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2])},
                    {-f[0], -f[1], -f[2], (f[0] * eye[0] + f[1] * eye[1] + f[2] * eye[2])},
                    {0, 0, 0, 1}};
  const double t = 1.0 / std::tan(0.5 * (double)fov_y_degrees * M_PI / 180.0);
  const double aspect = (double)width / (double)height;
  const double n = z_near, fr = z_far;
  double Pm[4][4] = {{t / aspect, 0, 0, 0}, {0, -t, 0, 0}, {0, 0, fr / (n - fr), n * fr / (n - fr)}, {0, 0, -1, 0}};
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 4; ++k) acc += Pm[r][k] * V[k][c];
      out->proj_view_matrix[c * 4 + r] = (float)acc;
      out->view_matrix[c * 4 + r] = (float)V[r][c];
    }
  return OIT_OK;
}

int oit_srgb_tables(float* thresholds256, float* decode256) {
  if (!thresholds256 || !decode256) return OIT_ERR_INVALID_ARGUMENT;
  oit::srgb_host_tables(thresholds256, decode256);
  return OIT_OK;
}

int oit_version(void) { return 100; }

}  // extern "C"
