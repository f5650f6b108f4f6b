/*
 * CPU oracle for the GB300 order-independent-transparency engine.
 * TEST INFRASTRUCTURE ONLY (see oit_oracle.h): the parity oracle for the
 * CUDA engine, never linked into or called by the product path.
 *
 * Build with -ffp-contract=off: the float32 raster/shading sequence below is
 * the specification the CUDA rasteriser reproduces bit for bit, so no
 * multiply-add may be fused except where fmaf() is written explicitly.
 *
 * Reference files cited as path:line within nvpro-samples/vk_order_independent_transparency.
 *
 * Two builds of this file (oracle/Makefile): the oracle (blending in FP64,
 * single-threaded) and, as a CPU baseline only, OR_FP32 + OpenMP: blending in
 * FP32 and the draws split over screen tiles (every triangle is set up, binned
 * into 32x32 tiles in primitive order, and each thread rasterises whole tiles,
 * so every pixel still sees its fragments in primitive order).
 */
#include "oit_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef OR_FP32
typedef float or_real;
#else
typedef double or_real;
#endif

#ifdef _OPENMP
#include <omp.h>
#define OR_OMP(x) _Pragma(x)
#else
#define OR_OMP(x)
#endif

#define EMPTY32 0xFFFFFFFFu
#define EMPTY64 0xFFFFFFFFFFFFFFFFull

/* ------------------------------------------------------------------------- */
/* sRGB conversions. shaderCommon.glsl:61-104 defines them with float pow;  */
/* the specification used here quantises with the exact threshold of each   */
/* 8-bit code (computed in double), so both CPU and GPU encode identically. */
/* ------------------------------------------------------------------------- */
static float g_thr[255];
static double g_dec[256];
static int g_tables_ready = 0;

static double enc_double(double c) {
  /* unPremultLinearToSRGB, shaderCommon.glsl:61-71 */
  if (c < 0.0031308) return c * 12.92;
  return pow(c, 1.0 / 2.4) * 1.055 - 0.055;
}

static float bits_to_float(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t float_to_bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static void init_tables(void) {
  if (g_tables_ready) return;
  for (int k = 0; k < 255; ++k) {
    double target = ((double)k + 0.5) / 255.0;
    uint32_t lo = 0, hi = 0x3F800000u; /* enc(1.0) = 1 >= target always */
    while (lo < hi) {
      uint32_t mid = lo + (hi - lo) / 2;
      if (enc_double((double)bits_to_float(mid)) >= target) hi = mid; else lo = mid + 1;
    }
    g_thr[k] = bits_to_float(lo);
  }
  for (int c = 0; c < 256; ++c) {
    /* unPremultSRGBToLinear, shaderCommon.glsl:83-93 */
    double s = (double)c / 255.0;
    g_dec[c] = (s < 0.04045) ? s / 12.92 : pow((s + 0.055) / 1.055, 2.4);
  }
  g_tables_ready = 1;
}

float or_srgb_threshold(int k) { init_tables(); return g_thr[k]; }
double or_srgb_decode(int code) { init_tables(); return g_dec[code & 255]; }

uint32_t or_srgb_encode(float c) {
  init_tables();
  /* number of thresholds <= c (NaN and negatives give 0) */
  int lo = 0, hi = 255;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (c >= g_thr[mid]) lo = mid + 1; else hi = mid;
  }
  return (uint32_t)lo;
}

static uint32_t encode_double(double c) {
  int lo = 0, hi = 255;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (c >= (double)g_thr[mid]) lo = mid + 1; else hi = mid;
  }
  return (uint32_t)lo;
}

static uint32_t unorm8(float x) {
  /* packUnorm4x8 component: round(clamp(x,0,1)*255) */
  x = (x > 0.0f) ? x : 0.0f;
  x = (x < 1.0f) ? x : 1.0f;
  return (uint32_t)rintf(x * 255.0f);
}

static uint32_t unorm8_double(double x) {
  x = (x > 0.0) ? x : 0.0;
  x = (x < 1.0) ? x : 1.0;
  return (uint32_t)rint(x * 255.0);
}

/* ------------------------------------------------------------------------- */
/* Frame state                                                               */
/* ------------------------------------------------------------------------- */
typedef struct { or_real r, g, b, a; } rgba_d;

struct or_frame {
  or_params p;
  int RW, RH;        /* render size */
  size_t P;          /* pixels of the render target */
  int S;             /* samples per pixel (msaa) */
  int coverage;      /* OIT_COVERAGE_SHADING, common.h:122 */
  int ss_layers;     /* sample-shading layers of the A-buffer (msaa or 1) */
  size_t E;          /* A-buffer elements (ss_layers * P) */
  int L;
  int rec_words;     /* words per Simple/Spinlock/Interlock record */
  uint32_t capacity; /* linked-list pool size in nodes (SceneData::linkedListAllocatedPerElement) */

  uint32_t* abuf; size_t abuf_words;
  uint32_t* aux;
  uint32_t* auxdepth;
  uint32_t counter;
  uint32_t* depth;   /* S*P opaque depth bits */
  rgba_d* color;     /* S*P colour target (premultiplied linear) */
  rgba_d* accum;     /* S*P WBOIT accumulation */
  or_real* reveal;   /* S*P WBOIT revealage */
  const uint32_t* ll_limit;
  uint32_t* ll_stored;
  uint32_t ll_alloc;
  uint64_t fragments;
};

static void* xcalloc(size_t n, size_t sz) {
  void* p = calloc(n ? n : 1, sz ? sz : 1);
  if (!p) abort();
  return p;
}

or_frame* or_frame_create(const or_params* p) {
  init_tables(); /* before any parallel region reads the tables */
  or_frame* f = (or_frame*)xcalloc(1, sizeof(or_frame));
  f->p = *p;
  int ss = p->supersample > 1 ? p->supersample : 1;
  f->RW = p->width * ss;
  f->RH = p->height * ss;
  f->P = (size_t)f->RW * (size_t)f->RH;
  f->S = p->msaa > 1 ? p->msaa : 1;
  f->coverage = (f->S > 1) && !p->sample_shading;
  f->ss_layers = p->sample_shading ? f->S : 1;
  f->E = (size_t)f->ss_layers * f->P;
  f->L = p->oit_layers;
  f->rec_words = f->coverage ? 4 : 2;
  /* A-buffer sizing, oit.cpp:100-163 */
  switch (p->algorithm) {
    case OR_SIMPLE: case OR_SPINLOCK: case OR_INTERLOCK:
      f->abuf_words = f->E * (size_t)f->L * (size_t)f->rec_words; break;
    case OR_LINKEDLIST:
      f->capacity = (uint32_t)((size_t)p->nodes_per_pixel * f->E);
      f->abuf_words = (size_t)f->capacity * (p->record_fp32 ? 8 : 4); break;
    case OR_LOOP: f->abuf_words = f->E * (size_t)f->L * 2; break;
    /* RGBA32F: a float4 payload block follows the 64-bit keys */
    case OR_LOOP64: f->abuf_words = f->E * (size_t)f->L * (p->record_fp32 ? 6 : 2); break;
    default: f->abuf_words = 0; break;
  }
  f->abuf = (uint32_t*)xcalloc(f->abuf_words, 4);
  f->aux = (uint32_t*)xcalloc(f->E, 4);
  f->auxdepth = (uint32_t*)xcalloc(f->E, 4);
  f->ll_stored = (uint32_t*)xcalloc(f->E, 4);
  f->depth = (uint32_t*)xcalloc((size_t)f->S * f->P, 4);
  f->color = (rgba_d*)xcalloc((size_t)f->S * f->P, sizeof(rgba_d));
  f->accum = (rgba_d*)xcalloc((size_t)f->S * f->P, sizeof(rgba_d));
  f->reveal = (or_real*)xcalloc((size_t)f->S * f->P, sizeof(or_real));
  or_begin(f);
  or_clear_transparent(f);
  return f;
}

void or_frame_destroy(or_frame* f) {
  if (!f) return;
  free(f->abuf); free(f->aux); free(f->auxdepth); free(f->ll_stored);
  free(f->depth); free(f->color); free(f->accum); free(f->reveal);
  free(f);
}

void or_begin(or_frame* f) {
  const float* bg = f->p.background;
  OR_OMP("omp parallel for schedule(static)")
  for (size_t i = 0; i < (size_t)f->S * f->P; ++i) {
    f->depth[i] = float_to_bits(1.0f);
    f->color[i].r = bg[0]; f->color[i].g = bg[1]; f->color[i].b = bg[2]; f->color[i].a = bg[3];
  }
}

void or_clear_transparent(or_frame* f) {
  /* oitRender.cpp:156-174 (Simple), 201-216 (LL), 242-265 (Loop), 303-311 (Loop64),
   * 337-356 (Spinlock/Interlock); WBOIT targets are cleared by its render pass
   * (oitRender.cpp:394-397). */
  memset(f->aux, 0, f->E * 4);
  OR_OMP("omp parallel for schedule(static)")
  for (size_t i = 0; i < f->E; ++i) f->auxdepth[i] = EMPTY32;
  memset(f->ll_stored, 0, f->E * 4);
  f->ll_alloc = 0;
  f->counter = 0;
  if (f->p.algorithm == OR_LOOP) {
    for (int s = 0; s < f->ss_layers; ++s)
      for (int i = 0; i < f->L; ++i)
        for (size_t px = 0; px < f->P; ++px)
          f->abuf[((size_t)s * 2 * f->L + i) * f->P + px] = EMPTY32;
  } else if (f->p.algorithm == OR_LOOP64) {
    OR_OMP("omp parallel for schedule(static)")
    for (size_t i = 0; i < f->abuf_words; ++i) f->abuf[i] = EMPTY32;
  }
  OR_OMP("omp parallel for schedule(static)")
  for (size_t i = 0; i < (size_t)f->S * f->P; ++i) {
    f->accum[i].r = f->accum[i].g = f->accum[i].b = f->accum[i].a = 0.0;
    f->reveal[i] = 1.0;
  }
  f->fragments = 0;
}

/* ------------------------------------------------------------------------- */
/* Raster specification                                                      */
/* ------------------------------------------------------------------------- */
/* Light direction normalize(vec3(-1,2,1)), shaderCommon.glsl:38, rounded to float. */
static const float LX = -0x1.a20bd8p-2f, LY = 0x1.a20bd8p-1f, LZ = 0x1.a20bd8p-2f;

/* Standard sample locations in 1/256 pixel (1x centre; Vulkan 4x and 8x patterns). */
static const int SAMPLE_1[1][2] = {{128, 128}};
static const int SAMPLE_4[4][2] = {{96, 32}, {224, 96}, {32, 160}, {160, 224}};
static const int SAMPLE_8[8][2] = {{144, 80}, {112, 176}, {208, 144}, {80, 48},
                                   {48, 208}, {16, 112}, {176, 240}, {240, 16}};

static const int (*sample_table(int S))[2] {
  return S == 8 ? SAMPLE_8 : (S == 4 ? SAMPLE_4 : SAMPLE_1);
}

typedef struct {
  int32_t X[3], Y[3];
  int tl[3];
  float z0, dz1, dz2, inv_area;
  float q[3];
  float nq[3][3];
  float vzq[3];
  float rgb[3];
  float alpha;
  uint32_t alpha_code;
  int bx0, by0, bx1, by1;
} tri_setup;

/* A clip-space vertex and the attributes the raster interpolates. */
typedef struct { float x, y, z, w, vz, n[3]; } clip_vert;

/* The vertex where edge a -> b crosses the near plane z = 0: attributes
 * interpolated linearly at t = za / (za - zb), z exactly 0. */
static clip_vert near_cut(const clip_vert* a, const clip_vert* b) {
  float t = a->z / (a->z - b->z);
  clip_vert r;
  r.x = fmaf(t, b->x - a->x, a->x);
  r.y = fmaf(t, b->y - a->y, a->y);
  r.z = 0.0f;
  r.w = fmaf(t, b->w - a->w, a->w);
  r.vz = fmaf(t, b->vz - a->vz, a->vz);
  for (int i = 0; i < 3; ++i) r.n[i] = fmaf(t, b->n[i] - a->n[i], a->n[i]);
  return r;
}

static int setup_half(const or_frame* f, const clip_vert* cv, const float* v0, int cull_back, tri_setup* T);

/* Vertex layout: utilities_vk.h:48-88 (pos.xyz, normal.xyz, color.rgba; 40 B).
 * Returns a bit mask of the triangle's halves that reach the raster: a
 * triangle wholly in front of the near plane has one (T[0]); one the plane
 * crosses is clipped (Sutherland-Hodgman against z = 0 in clip space, over
 * the edges 0->1, 1->2, 2->0) into a triangle (T[0]) or a quad split into the
 * fan (0, 1, 2) = T[0] and (0, 2, 3) = T[1]. */
static int setup_triangle(const or_frame* f, const float* pv, const float* view,
                          const float* vertices, const uint32_t* indices, uint32_t t,
                          int cull_back, tri_setup T[2]) {
  clip_vert cv[3];
  const float* v0 = vertices + 10 * (size_t)indices[3 * (size_t)t];
  for (int k = 0; k < 3; ++k) {
    const float* v = vertices + 10 * (size_t)indices[3 * (size_t)t + k];
    float x = v[0], y = v[1], z = v[2];
    /* object.vert.glsl:34-35: gl_Position = projView * pos; depth = (view * pos).z */
    cv[k].x = fmaf(pv[0], x, fmaf(pv[4], y, fmaf(pv[8], z, pv[12])));
    cv[k].y = fmaf(pv[1], x, fmaf(pv[5], y, fmaf(pv[9], z, pv[13])));
    cv[k].z = fmaf(pv[2], x, fmaf(pv[6], y, fmaf(pv[10], z, pv[14])));
    cv[k].w = fmaf(pv[3], x, fmaf(pv[7], y, fmaf(pv[11], z, pv[15])));
    cv[k].vz = fmaf(view[2], x, fmaf(view[6], y, fmaf(view[10], z, view[14])));
    cv[k].n[0] = v[3]; cv[k].n[1] = v[4]; cv[k].n[2] = v[5];
  }
  int nin = (cv[0].z >= 0.0f) + (cv[1].z >= 0.0f) + (cv[2].z >= 0.0f);
  if (nin == 3 || nin == 0) return setup_half(f, cv, v0, cull_back, &T[0]);
  clip_vert poly[4];
  int n = 0;
  for (int k = 0; k < 3; ++k) {
    const clip_vert* a = &cv[k];
    const clip_vert* b = &cv[(k + 1) % 3];
    int ina = a->z >= 0.0f, inb = b->z >= 0.0f;
    if (ina) poly[n++] = *a;
    if (ina != inb) poly[n++] = near_cut(a, b);
  }
  int mask = setup_half(f, poly, v0, cull_back, &T[0]);
  if (n == 4) {
    clip_vert second[3] = {poly[0], poly[2], poly[3]};
    mask |= setup_half(f, second, v0, cull_back, &T[1]) << 1;
  }
  return mask;
}

/* One triangle of clip-space vertices: the 0 <= z <= w, w > 0 test (far
 * plane and w <= 0: dropped), projection, snap, orientation, bbox, record. */
static int setup_half(const or_frame* f, const clip_vert* cv, const float* v0, int cull_back, tri_setup* T) {
  float cx[3], cy[3], cz[3], cw[3], vz[3], n[3][3];
  for (int k = 0; k < 3; ++k) {
    cx[k] = cv[k].x; cy[k] = cv[k].y; cz[k] = cv[k].z; cw[k] = cv[k].w; vz[k] = cv[k].vz;
    n[k][0] = cv[k].n[0]; n[k][1] = cv[k].n[1]; n[k][2] = cv[k].n[2];
  }
  for (int k = 0; k < 3; ++k)
    if (!(cw[k] > 0.0f) || !(cz[k] >= 0.0f) || !(cz[k] <= cw[k])) return 0;
  const float halfW = 0.5f * (float)f->RW, halfH = 0.5f * (float)f->RH;
  float zz[3], q[3];
  for (int k = 0; k < 3; ++k) {
    q[k] = 1.0f / cw[k];
    float nx = cx[k] * q[k], ny = cy[k] * q[k];
    zz[k] = cz[k] * q[k];
    float sx = fmaf(nx, halfW, halfW), sy = fmaf(ny, halfH, halfH);
    if (!(fabsf(sx) < 16384.0f) || !(fabsf(sy) < 16384.0f)) return 0;
    T->X[k] = (int32_t)rintf(sx * 256.0f);
    T->Y[k] = (int32_t)rintf(sy * 256.0f);
  }
  int64_t area = (int64_t)(T->X[1] - T->X[0]) * (int64_t)(T->Y[2] - T->Y[0]) -
                 (int64_t)(T->Y[1] - T->Y[0]) * (int64_t)(T->X[2] - T->X[0]);
  if (area == 0) return 0;
  /* Normalise orientation so that area > 0 by swapping vertices 1 and 2. */
  int order[3] = {0, 1, 2};
  if (area > 0) {
    /* area > 0 is clockwise on the y-down framebuffer: a back face for
     * VK_FRONT_FACE_COUNTER_CLOCKWISE (main.cpp:520-525). */
    if (cull_back) return 0;
  } else {
    area = -area;
    order[1] = 2; order[2] = 1;
  }
  int32_t X[3], Y[3];
  float z[3], qq[3], vzz[3], nn[3][3];
  for (int k = 0; k < 3; ++k) {
    int o = order[k];
    X[k] = T->X[o]; Y[k] = T->Y[o]; z[k] = zz[o]; qq[k] = q[o]; vzz[k] = vz[o];
    nn[k][0] = n[o][0]; nn[k][1] = n[o][1]; nn[k][2] = n[o][2];
  }
  for (int k = 0; k < 3; ++k) { T->X[k] = X[k]; T->Y[k] = Y[k]; }
  /* top-left rule: edge i runs from vertex (i+1)%3 to (i+2)%3 */
  for (int i = 0; i < 3; ++i) {
    int a = (i + 1) % 3, b = (i + 2) % 3;
    int32_t dx = X[b] - X[a], dy = Y[b] - Y[a];
    T->tl[i] = (dy < 0) || (dy == 0 && dx > 0);
  }
  int32_t minX = X[0], maxX = X[0], minY = Y[0], maxY = Y[0];
  for (int k = 1; k < 3; ++k) {
    if (X[k] < minX) minX = X[k];
    if (X[k] > maxX) maxX = X[k];
    if (Y[k] < minY) minY = Y[k];
    if (Y[k] > maxY) maxY = Y[k];
  }
  T->bx0 = minX >> 8; T->by0 = minY >> 8; T->bx1 = maxX >> 8; T->by1 = maxY >> 8;
  if (T->bx0 < 0) T->bx0 = 0;
  if (T->by0 < 0) T->by0 = 0;
  if (T->bx1 > f->RW - 1) T->bx1 = f->RW - 1;
  if (T->by1 > f->RH - 1) T->by1 = f->RH - 1;
  if (T->bx0 > T->bx1 || T->by0 > T->by1) return 0;
  T->z0 = z[0];
  T->dz1 = z[1] - z[0];
  T->dz2 = z[2] - z[0];
  T->inv_area = 1.0f / (float)area;
  for (int k = 0; k < 3; ++k) {
    T->q[k] = qq[k];
    T->nq[k][0] = nn[k][0] * qq[k];
    T->nq[k][1] = nn[k][1] * qq[k];
    T->nq[k][2] = nn[k][2] * qq[k];
    T->vzq[k] = vzz[k] * qq[k];
  }
  /* Colour is flat per triangle (provoking vertex 0): the sphere scenes give
   * every vertex of an object the same colour. */
  T->rgb[0] = v0[6]; T->rgb[1] = v0[7]; T->rgb[2] = v0[8];
  /* shading(), shaderCommon.glsl:48-56: alpha = clamp(alphaMin + a*alphaWidth, 0, 1) */
  float a = fmaf(v0[9], f->p.alpha_width, f->p.alpha_min);
  a = (a > 0.0f) ? a : 0.0f;
  a = (a < 1.0f) ? a : 1.0f;
  T->alpha = a;
  T->alpha_code = unorm8(a);
  return 1;
}

static inline void edges_at(const tri_setup* T, int32_t px, int32_t py, int64_t e[3]) {
  e[0] = (int64_t)(T->X[2] - T->X[1]) * (int64_t)(py - T->Y[1]) -
         (int64_t)(T->Y[2] - T->Y[1]) * (int64_t)(px - T->X[1]);
  e[1] = (int64_t)(T->X[0] - T->X[2]) * (int64_t)(py - T->Y[2]) -
         (int64_t)(T->Y[0] - T->Y[2]) * (int64_t)(px - T->X[2]);
  e[2] = (int64_t)(T->X[1] - T->X[0]) * (int64_t)(py - T->Y[0]) -
         (int64_t)(T->Y[1] - T->Y[0]) * (int64_t)(px - T->X[0]);
}

static inline int inside(const tri_setup* T, const int64_t e[3]) {
  for (int i = 0; i < 3; ++i)
    if (!(e[i] > 0 || (e[i] == 0 && T->tl[i]))) return 0;
  return 1;
}

static inline float depth_at(const tri_setup* T, const int64_t e[3]) {
  float b1 = (float)e[1] * T->inv_area;
  float b2 = (float)e[2] * T->inv_area;
  float z = fmaf(b2, T->dz2, fmaf(b1, T->dz1, T->z0));
  z = (z > 0.0f) ? z : 0.0f;
  z = (z < 1.0f) ? z : 1.0f;
  return z;
}

typedef struct {
  uint32_t packed;   /* packUnorm4x8(unPremultLinearToSRGB(shading)) */
  uint32_t depth;    /* floatBitsToUint(gl_FragCoord.z) */
  uint32_t mask;     /* post-depth coverage (coverage shading) */
  float rgba[4];     /* shading() result: linear, unpremultiplied */
  float view_z;      /* Interpolants::depth (view-space z) */
} frag_t;

/* Gooch shading at a shading point with edge values e (shaderCommon.glsl:36-56). */
static void shade(const tri_setup* T, const int64_t e[3], float rgb_out[3], float* view_z) {
  float b0 = (float)e[0] * T->inv_area;
  float b1 = (float)e[1] * T->inv_area;
  float b2 = (float)e[2] * T->inv_area;
  float nx = fmaf(b2, T->nq[2][0], fmaf(b1, T->nq[1][0], b0 * T->nq[0][0]));
  float ny = fmaf(b2, T->nq[2][1], fmaf(b1, T->nq[1][1], b0 * T->nq[0][1]));
  float nz = fmaf(b2, T->nq[2][2], fmaf(b1, T->nq[1][2], b0 * T->nq[0][2]));
  float len2 = fmaf(nz, nz, fmaf(ny, ny, nx * nx));
  float d = fmaf(nz, LZ, fmaf(ny, LY, nx * LX));
  float c = (len2 > 0.0f) ? d / sqrtf(len2) : 0.0f;
  float warmth = fmaf(c, 0.5f, 0.5f);
  rgb_out[0] = T->rgb[0] * warmth;
  rgb_out[1] = T->rgb[1] * fmaf(0.75f, warmth, 0.25f);
  rgb_out[2] = T->rgb[2] * fmaf(0.25f, warmth, 0.75f);
  if (view_z) {
    float num = fmaf(b2, T->vzq[2], fmaf(b1, T->vzq[1], b0 * T->vzq[0]));
    float den = fmaf(b2, T->q[2], fmaf(b1, T->q[1], b0 * T->q[0]));
    *view_z = num / den;
  }
}

/* ------------------------------------------------------------------------- */
/* Blending helpers                                                          */
/* ------------------------------------------------------------------------- */
static rgba_d premult_float(const float c[4]) {
  rgba_d r = {(or_real)c[0] * c[3], (or_real)c[1] * c[3], (or_real)c[2] * c[3], (or_real)c[3]};
  return r;
}

static rgba_d decode_packed(uint32_t packed) {
  /* unpackUnorm4x8 + unPremultSRGBToLinear, shaderCommon.glsl:117-124 (before premultiply) */
  rgba_d r = {g_dec[packed & 255], g_dec[(packed >> 8) & 255], g_dec[(packed >> 16) & 255],
              (or_real)((packed >> 24) & 255) / (or_real)255.0};
  return r;
}

static rgba_d premult(rgba_d c) {
  rgba_d r = {c.r * c.a, c.g * c.a, c.b * c.a, c.a};
  return r;
}

/* doBlend: color = color over base (shaderCommon.glsl:108-112) */
static void do_blend(rgba_d* color, rgba_d base) {
  or_real k = (or_real)1.0 - color->a;
  color->r += k * base.r; color->g += k * base.g; color->b += k * base.b; color->a += k * base.a;
}

/* doBlendPacked (shaderCommon.glsl:117-124) */
static void do_blend_packed(rgba_d* color, uint32_t packed) {
  do_blend(color, premult(decode_packed(packed)));
}

/* Hardware blend ONE, ONE_MINUS_SRC_ALPHA (main.cpp:548-558): dst = src + (1-src.a) dst */
static void rop_premultiplied(rgba_d* dst, rgba_d src) {
  or_real k = (or_real)1.0 - src.a;
  dst->r = src.r + k * dst->r; dst->g = src.g + k * dst->g;
  dst->b = src.b + k * dst->b; dst->a = src.a + k * dst->a;
}

/* Writes the fragment output colour into the samples it covers. */
static void tail_out(or_frame* f, size_t pixel, int sample, uint32_t cover, rgba_d src) {
  if (src.r == 0.0 && src.g == 0.0 && src.b == 0.0 && src.a == 0.0) return;
  if (f->p.sample_shading) {
    rop_premultiplied(&f->color[(size_t)sample * f->P + pixel], src);
  } else {
    for (int s = 0; s < f->S; ++s)
      if (cover & (1u << s)) rop_premultiplied(&f->color[(size_t)s * f->P + pixel], src);
  }
}

/* ------------------------------------------------------------------------- */
/* Per-fragment algorithm bodies (COLOR / DEPTH passes)                       */
/* ------------------------------------------------------------------------- */
static inline uint32_t* rec_ptr(or_frame* f, size_t elem_s, size_t pixel, int layer) {
  /* listPos = viewSize*OIT_LAYERS*sampleID + pixel; record at listPos + layer*viewSize */
  size_t r = (elem_s * (size_t)f->L + (size_t)layer) * f->P + pixel;
  return f->abuf + r * (size_t)f->rec_words;
}

static void store_rec(or_frame* f, uint32_t* dst, const frag_t* fr) {
  dst[0] = fr->packed;
  dst[1] = fr->depth;
  if (f->rec_words == 4) { dst[2] = fr->mask; dst[3] = 0; }
}

static rgba_d zero_rgba(void) { rgba_d z = {0, 0, 0, 0}; return z; }

/* oitSimple.frag.glsl:50-91 */
static void frag_simple(or_frame* f, size_t pixel, int s, uint32_t cover, const frag_t* fr) {
  size_t e = (size_t)s * f->P + pixel;
  uint32_t old = f->aux[e]++;
  if (old < (uint32_t)f->L) {
    store_rec(f, rec_ptr(f, s, pixel, (int)old), fr);
  } else if (f->p.tail_blend) {
    tail_out(f, pixel, s, cover, premult_float(fr->rgba));
  }
}

/* oitLinkedList.frag.glsl:51-85 */
static void frag_linkedlist(or_frame* f, size_t pixel, int s, uint32_t cover, const frag_t* fr) {
  size_t e = (size_t)s * f->P + pixel;
  uint32_t newOffset;
  OR_OMP("omp atomic capture")
  newOffset = f->counter++;
  newOffset += 1u;
  int overflow = newOffset >= f->capacity;
  if (f->ll_limit) {
    /* replay: the caller decides how many nodes each element got; nodes are
     * numbered in this oracle's own order */
    overflow = f->ll_stored[e] >= f->ll_limit[e];
    if (!overflow) {
      OR_OMP("omp atomic capture")
      newOffset = ++f->ll_alloc;
    }
    if (newOffset >= f->capacity) overflow = 1;
  }
  if (overflow) {
    if (f->p.tail_blend) tail_out(f, pixel, s, cover, premult_float(fr->rgba));
    return;
  }
  f->ll_stored[e]++;
  uint32_t oldOffset = f->aux[e];
  f->aux[e] = newOffset;
  if (f->p.record_fp32) {
    /* RGBA32F node: linear unpremultiplied colour, depth, mask, next, 0 */
    uint32_t* n = f->abuf + (size_t)newOffset * 8;
    for (int k = 0; k < 4; ++k) n[k] = float_to_bits(fr->rgba[k]);
    n[4] = fr->depth; n[5] = f->coverage ? fr->mask : 0u; n[6] = oldOffset; n[7] = 0;
    return;
  }
  uint32_t* n = f->abuf + (size_t)newOffset * 4;
  n[0] = fr->packed; n[1] = fr->depth; n[2] = f->coverage ? fr->mask : 0u; n[3] = oldOffset;
}

/* oitLoop.frag.glsl:57-100 (DEPTH pass) */
static void frag_loop_depth(or_frame* f, size_t pixel, int s, const frag_t* fr) {
  size_t listPos = (size_t)s * 2 * f->L * f->P + pixel;
  const int L = f->L;
  uint32_t zcur = fr->depth;
  int i = 0;
  if (zcur > f->abuf[listPos + (size_t)(L - 1) * f->P]) return;
  if (zcur > f->abuf[listPos + (size_t)(L / 2) * f->P]) i = L / 2;
  for (; i < L; ++i) {
    uint32_t* slot = &f->abuf[listPos + (size_t)i * f->P];
    uint32_t ztest = *slot;
    if (zcur < ztest) *slot = zcur; /* atomicMin */
    if (ztest == EMPTY32 || ztest == zcur) break;
    zcur = ztest > zcur ? ztest : zcur;
  }
}

/* oitLoop.frag.glsl:120-173 (COLOR pass) */
static void frag_loop_color(or_frame* f, size_t pixel, int s, uint32_t cover, const frag_t* fr) {
  size_t listPos = (size_t)s * 2 * f->L * f->P + pixel;
  const int L = f->L;
  uint32_t zcur = fr->depth;
  if (f->abuf[listPos + (size_t)(L - 1) * f->P] < zcur) {
    if (f->p.tail_blend) tail_out(f, pixel, s, cover, premult_float(fr->rgba));
    return;
  }
  int start = 0, end = L - 1;
  while (start < end) {
    int mid = (start + end) / 2;
    uint32_t ztest = f->abuf[listPos + (size_t)mid * f->P];
    if (ztest < zcur) start = mid + 1; else end = mid;
  }
  f->abuf[listPos + (size_t)(L + start) * f->P] = fr->packed;
}

/* oitLoop64.frag.glsl:65-141 */
static void frag_loop64(or_frame* f, size_t pixel, int s, uint32_t cover, const frag_t* fr) {
  const int L = f->L;
  size_t listPos = (size_t)s * L * f->P + pixel;
  uint64_t* ab = (uint64_t*)f->abuf; /* little-endian: low word = colour, high word = depth */
  float* pay = f->p.record_fp32 ? (float*)(f->abuf + f->E * (size_t)L * 2) : NULL;
  uint64_t zcur = ((uint64_t)fr->depth << 32) | fr->packed;
  float pcur[4] = {fr->rgba[0], fr->rgba[1], fr->rgba[2], fr->rgba[3]};
  int i = 0, canInsert = 1;
  uint64_t pretest = ab[listPos + (size_t)(L - 1) * f->P];
  if (zcur > pretest) {
    canInsert = 0;
  } else {
    pretest = ab[listPos + (size_t)(L / 2) * f->P];
    if (zcur > pretest) i = L / 2;
  }
  int evict = 1;
  if (canInsert) {
    for (; i < L; ++i) {
      uint64_t* slot = &ab[listPos + (size_t)i * f->P];
      uint64_t ztest = *slot;
      if (zcur < ztest) { /* atomicMin; a float payload moves with its key */
        *slot = zcur;
        if (pay) {
          float* ps = pay + 4 * (listPos + (size_t)i * f->P);
          for (int k = 0; k < 4; ++k) { float t = ps[k]; ps[k] = pcur[k]; pcur[k] = t; }
        }
      }
      if (ztest == EMPTY64) { evict = 0; break; }
      zcur = ztest > zcur ? ztest : zcur;
    }
  }
  if (evict && f->p.tail_blend)
    tail_out(f, pixel, s, cover, pay ? premult_float(pcur) : premult(decode_packed((uint32_t)(zcur & 0xFFFFFFFFu))));
}

/* oitSpinlock.frag.glsl:49-129 and oitInterlock.frag.glsl:90-152. Both run
 * here in primitive order, which is one of the orders the reference allows
 * for Spinlock and the order it guarantees for ordered Interlock. */
static void frag_lock(or_frame* f, size_t pixel, int s, uint32_t cover, const frag_t* fr) {
  size_t e = (size_t)s * f->P + pixel;
  const int L = f->L;
  rgba_d color = {fr->rgba[0], fr->rgba[1], fr->rgba[2], fr->rgba[3]};
  int own = 1;
  if (fr->depth <= f->auxdepth[e]) {
    uint32_t oldCounter = f->aux[e];
    f->aux[e] = oldCounter + 1;
    if (oldCounter < (uint32_t)L) {
      store_rec(f, rec_ptr(f, s, pixel, (int)oldCounter), fr);
      color = zero_rgba();
      own = 0;
    } else {
      int furthest = 0;
      uint32_t maxDepth = 0;
      for (int i = 0; i < L; ++i) {
        uint32_t d = rec_ptr(f, s, pixel, i)[1];
        if (d > maxDepth) { maxDepth = d; furthest = i; }
      }
      if (maxDepth > fr->depth) {
        uint32_t* r = rec_ptr(f, s, pixel, furthest);
        color = decode_packed(r[0]);
        own = 0;
        store_rec(f, r, fr);
        f->auxdepth[e] = maxDepth;
      }
    }
  }
  (void)own;
  if (f->p.tail_blend) tail_out(f, pixel, s, cover, premult(color));
}

/* oitWeighted.frag.glsl:53-79; blend state main.cpp:559-577 */
static void frag_weighted(or_frame* f, size_t pixel, uint32_t cover, const frag_t* fr) {
  rgba_d c = premult_float(fr->rgba);
  or_real depthZ = -(or_real)fr->view_z * (or_real)10.0;
  or_real x = depthZ / (or_real)200.0;
  or_real distWeight = (or_real)0.03 / ((or_real)1e-5 + x * x * x * x);
  distWeight = distWeight < 1e-2 ? 1e-2 : (distWeight > 3e3 ? 3e3 : distWeight);
  or_real m = c.r > c.g ? c.r : c.g;
  or_real m2 = c.b > c.a ? c.b : c.a;
  m = m > m2 ? m : m2;
  or_real alphaWeight = m * (or_real)40.0 + (or_real)0.01;
  alphaWeight = alphaWeight < 1.0 ? alphaWeight : 1.0;
  alphaWeight *= alphaWeight;
  or_real w = alphaWeight * distWeight;
  for (int s = 0; s < f->S; ++s) {
    if (!(cover & (1u << s))) continue;
    size_t i = (size_t)s * f->P + pixel;
    f->accum[i].r += c.r * w; f->accum[i].g += c.g * w;
    f->accum[i].b += c.b * w; f->accum[i].a += c.a * w;
    f->reveal[i] *= (1.0 - c.a);
  }
}

/* The callers count fragments (Loop32 sees each twice: counted in its colour pass). */
static void dispatch_fragment(or_frame* f, size_t pixel, int s, uint32_t cover, const frag_t* fr, int loop_pass) {
  switch (f->p.algorithm) {
    case OR_SIMPLE: frag_simple(f, pixel, s, cover, fr); break;
    case OR_LINKEDLIST: frag_linkedlist(f, pixel, s, cover, fr); break;
    case OR_LOOP:
      if (loop_pass == 0) frag_loop_depth(f, pixel, s, fr); else frag_loop_color(f, pixel, s, cover, fr);
      break;
    case OR_LOOP64: frag_loop64(f, pixel, s, cover, fr); break;
    case OR_SPINLOCK: case OR_INTERLOCK: frag_lock(f, pixel, s, cover, fr); break;
    case OR_WEIGHTED: frag_weighted(f, pixel, cover, fr); break;
    default: break;
  }
}

void or_inject_fragments(or_frame* f, int n, const int32_t* xy, const int32_t* sample,
                         const float* rgba, const float* depth, const uint32_t* mask,
                         const float* view_z) {
  int passes = f->p.algorithm == OR_LOOP ? 2 : 1;
  for (int pass = 0; pass < passes; ++pass) {
    int loop_pass = (f->p.algorithm == OR_LOOP) ? pass : 1;
    for (int i = 0; i < n; ++i) {
      const float* c = rgba + 4 * (size_t)i;
      frag_t fr;
      fr.rgba[0] = c[0]; fr.rgba[1] = c[1]; fr.rgba[2] = c[2]; fr.rgba[3] = c[3];
      fr.packed = or_srgb_encode(c[0]) | (or_srgb_encode(c[1]) << 8) |
                  (or_srgb_encode(c[2]) << 16) | (unorm8(c[3]) << 24);
      fr.depth = float_to_bits(depth[i]);
      uint32_t m = mask ? mask[i] : 1u;
      fr.mask = f->coverage ? m : 0u;
      fr.view_z = view_z ? view_z[i] : -1.0f;
      int s = sample ? sample[i] : 0;
      size_t pixel = (size_t)xy[2 * (size_t)i + 1] * f->RW + (size_t)xy[2 * (size_t)i];
      uint32_t cover = f->p.sample_shading ? (1u << s) : (f->coverage ? m : 1u);
      dispatch_fragment(f, pixel, f->p.sample_shading ? s : 0, cover, &fr, loop_pass);
      if (loop_pass == 1) f->fragments++;
    }
  }
}

/* Rasterises one triangle over the pixels of [x0, x1] x [y0, y1] and calls
 * the fragment body for each fragment; returns the fragments it counts. */
static uint64_t raster_transparent(or_frame* f, const tri_setup* T, int loop_pass, int x0, int y0, int x1, int y1) {
  const int S = f->S;
  const int (*st)[2] = sample_table(S);
  uint64_t n = 0;
  const int ya = T->by0 > y0 ? T->by0 : y0, yb = T->by1 < y1 ? T->by1 : y1;
  const int xa = T->bx0 > x0 ? T->bx0 : x0, xb = T->bx1 < x1 ? T->bx1 : x1;
  for (int py = ya; py <= yb; ++py) {
    for (int px = xa; px <= xb; ++px) {
      size_t pixel = (size_t)py * f->RW + px;
      int32_t bx = px * 256, by = py * 256;
      /* WBOIT never uses per-sample A-buffers: its COLOR shader does not read
       * gl_SampleID (oitColorDepthDefines.glsl:49), so it shades per pixel */
      if (f->p.sample_shading && f->p.algorithm != OR_WEIGHTED) {
        for (int s = 0; s < S; ++s) {
          int64_t e[3];
          edges_at(T, bx + st[s][0], by + st[s][1], e);
          if (!inside(T, e)) continue;
          float z = depth_at(T, e);
          uint32_t zb = float_to_bits(z);
          if (!(zb < f->depth[(size_t)s * f->P + pixel])) continue; /* early depth LESS */
          frag_t fr;
          float rgb[3];
          shade(T, e, rgb, &fr.view_z);
          fr.rgba[0] = rgb[0]; fr.rgba[1] = rgb[1]; fr.rgba[2] = rgb[2]; fr.rgba[3] = T->alpha;
          fr.packed = or_srgb_encode(rgb[0]) | (or_srgb_encode(rgb[1]) << 8) |
                      (or_srgb_encode(rgb[2]) << 16) | (T->alpha_code << 24);
          fr.depth = zb;
          fr.mask = 0;
          dispatch_fragment(f, pixel, s, 1u << s, &fr, loop_pass);
          n += loop_pass == 1;
        }
      } else {
        uint32_t mask = 0;
        for (int s = 0; s < S; ++s) {
          int64_t e[3];
          edges_at(T, bx + st[s][0], by + st[s][1], e);
          if (!inside(T, e)) continue;
          uint32_t zb = float_to_bits(depth_at(T, e));
          if (zb < f->depth[(size_t)s * f->P + pixel]) mask |= 1u << s;
        }
        if (!mask) continue;
        int64_t e[3];
        edges_at(T, bx + 128, by + 128, e);
        frag_t fr;
        float rgb[3];
        shade(T, e, rgb, &fr.view_z);
        fr.rgba[0] = rgb[0]; fr.rgba[1] = rgb[1]; fr.rgba[2] = rgb[2]; fr.rgba[3] = T->alpha;
        fr.packed = or_srgb_encode(rgb[0]) | (or_srgb_encode(rgb[1]) << 8) |
                    (or_srgb_encode(rgb[2]) << 16) | (T->alpha_code << 24);
        fr.depth = float_to_bits(depth_at(T, e));
        fr.mask = f->coverage ? mask : 0u;
        dispatch_fragment(f, pixel, 0, mask, &fr, loop_pass);
        n += loop_pass == 1;
      }
    }
  }
  return n;
}

#ifdef _OPENMP
/* Tile-parallel draws: every triangle set up once, then binned into
 * kOrTile x kOrTile pixel tiles in primitive order (CSR lists). */
enum { kOrTile = 32 };
typedef struct {
  tri_setup* T;      /* two slots per triangle: its halves */
  unsigned char* ok; /* bit mask of the triangle's halves */
  uint32_t* start; /* [tiles + 1] */
  uint32_t* list;  /* triangle slots, primitive order per tile */
  int tx, ty;
} or_bins;

static void bins_free(or_bins* b) {
  free(b->T);
  free(b->ok);
  free(b->start);
  free(b->list);
}

static void bins_build(const or_frame* f, const float* pv, const float* view, const float* vertices,
                       const uint32_t* indices, uint32_t first, uint32_t count, int opaque, or_bins* b) {
  b->T = (tri_setup*)xcalloc(2 * (size_t)(count ? count : 1), sizeof(tri_setup));
  b->ok = (unsigned char*)xcalloc(count ? count : 1, 1);
  OR_OMP("omp parallel for schedule(static)")
  for (int64_t i = 0; i < (int64_t)count; ++i)
    b->ok[i] = (unsigned char)setup_triangle(f, pv, view, vertices, indices, first + (uint32_t)i, opaque, &b->T[2 * i]);
  b->tx = (f->RW + kOrTile - 1) / kOrTile;
  b->ty = (f->RH + kOrTile - 1) / kOrTile;
  const size_t nt = (size_t)b->tx * b->ty;
  b->start = (uint32_t*)xcalloc(nt + 1, sizeof(uint32_t));
  for (uint32_t i = 0; i < 2 * count; ++i) {
    if (!((b->ok[i >> 1] >> (i & 1)) & 1)) continue;
    const tri_setup* T = &b->T[i];
    for (int y = T->by0 / kOrTile; y <= T->by1 / kOrTile; ++y)
      for (int x = T->bx0 / kOrTile; x <= T->bx1 / kOrTile; ++x) b->start[(size_t)y * b->tx + x + 1]++;
  }
  for (size_t k = 0; k < nt; ++k) b->start[k + 1] += b->start[k];
  b->list = (uint32_t*)xcalloc(b->start[nt] ? b->start[nt] : 1, sizeof(uint32_t));
  uint32_t* cur = (uint32_t*)xcalloc(nt ? nt : 1, sizeof(uint32_t));
  memcpy(cur, b->start, nt * sizeof(uint32_t));
  for (uint32_t i = 0; i < 2 * count; ++i) {
    if (!((b->ok[i >> 1] >> (i & 1)) & 1)) continue;
    const tri_setup* T = &b->T[i];
    for (int y = T->by0 / kOrTile; y <= T->by1 / kOrTile; ++y)
      for (int x = T->bx0 / kOrTile; x <= T->bx1 / kOrTile; ++x) b->list[cur[(size_t)y * b->tx + x]++] = i;
  }
  free(cur);
}
#endif

void or_draw_transparent(or_frame* f, const float* pv, const float* view, const float* vertices,
                         const uint32_t* indices, uint32_t first, uint32_t count) {
  int passes = f->p.algorithm == OR_LOOP ? 2 : 1;
#ifdef _OPENMP
  or_bins b;
  bins_build(f, pv, view, vertices, indices, first, count, 0, &b);
  uint64_t frags = 0;
  OR_OMP("omp parallel for schedule(dynamic, 1) reduction(+ : frags)")
  for (int64_t k = 0; k < (int64_t)b.tx * b.ty; ++k) {
    const int x0 = (int)(k % b.tx) * kOrTile, y0 = (int)(k / b.tx) * kOrTile;
    for (int pass = 0; pass < passes; ++pass) {
      int loop_pass = (f->p.algorithm == OR_LOOP) ? pass : 1;
      for (uint32_t j = b.start[k]; j < b.start[k + 1]; ++j)
        frags += raster_transparent(f, &b.T[b.list[j]], loop_pass, x0, y0, x0 + kOrTile - 1, y0 + kOrTile - 1);
    }
  }
  f->fragments += frags;
  bins_free(&b);
#else
  for (int pass = 0; pass < passes; ++pass) {
    int loop_pass = (f->p.algorithm == OR_LOOP) ? pass : 1;
    for (uint32_t t = first; t < first + count; ++t) {
      tri_setup T[2];
      const int halves = setup_triangle(f, pv, view, vertices, indices, t, 0, T);
      for (int h = 0; h < 2; ++h)
        if ((halves >> h) & 1) f->fragments += raster_transparent(f, &T[h], loop_pass, 0, 0, f->RW - 1, f->RH - 1);
    }
  }
#endif
}

static void raster_opaque(or_frame* f, const tri_setup* T, int x0, int y0, int x1, int y1) {
  const int S = f->S;
  const int (*st)[2] = sample_table(S);
  const int ya = T->by0 > y0 ? T->by0 : y0, yb = T->by1 < y1 ? T->by1 : y1;
  const int xa = T->bx0 > x0 ? T->bx0 : x0, xb = T->bx1 < x1 ? T->bx1 : x1;
  for (int py = ya; py <= yb; ++py) {
    for (int px = xa; px <= xb; ++px) {
      size_t pixel = (size_t)py * f->RW + px;
      int32_t bx = px * 256, by = py * 256;
      int shaded = 0;
      rgba_d col = {0, 0, 0, 1};
      for (int s = 0; s < S; ++s) {
        int64_t e[3];
        edges_at(T, bx + st[s][0], by + st[s][1], e);
        if (!inside(T, e)) continue;
        uint32_t zb = float_to_bits(depth_at(T, e));
        size_t i = (size_t)s * f->P + pixel;
        if (!(zb < f->depth[i])) continue;
        if (!shaded) {
          int64_t ec[3];
          edges_at(T, bx + 128, by + 128, ec);
          float rgb[3];
          shade(T, ec, rgb, NULL);
          col.r = rgb[0]; col.g = rgb[1]; col.b = rgb[2]; col.a = 1.0;
          shaded = 1;
        }
        f->depth[i] = zb;
        f->color[i] = col;
      }
    }
  }
}

/* opaque.frag.glsl:30-35 with depth LESS + write (main.cpp:542-547) */
void or_draw_opaque(or_frame* f, const float* pv, const float* view, const float* vertices,
                    const uint32_t* indices, uint32_t first, uint32_t count) {
#ifdef _OPENMP
  or_bins b;
  bins_build(f, pv, view, vertices, indices, first, count, 1, &b);
  OR_OMP("omp parallel for schedule(dynamic, 1)")
  for (int64_t k = 0; k < (int64_t)b.tx * b.ty; ++k) {
    const int x0 = (int)(k % b.tx) * kOrTile, y0 = (int)(k / b.tx) * kOrTile;
    for (uint32_t j = b.start[k]; j < b.start[k + 1]; ++j)
      raster_opaque(f, &b.T[b.list[j]], x0, y0, x0 + kOrTile - 1, y0 + kOrTile - 1);
  }
  bins_free(&b);
#else
  for (uint32_t t = first; t < first + count; ++t) {
    tri_setup T[2];
    const int halves = setup_triangle(f, pv, view, vertices, indices, t, 1, T);
    for (int h = 0; h < 2; ++h)
      if ((halves >> h) & 1) raster_opaque(f, &T[h], 0, 0, f->RW - 1, f->RH - 1);
  }
#endif
}

/* ------------------------------------------------------------------------- */
/* COMPOSITE                                                                 */
/* ------------------------------------------------------------------------- */
typedef struct { uint32_t r, g, b; } rec3; /* (packed colour, depth bits, mask) */

static int depth_ge(uint32_t a, uint32_t b) { return bits_to_float(a) >= bits_to_float(b); }
static int depth_lt(uint32_t a, uint32_t b) { return bits_to_float(a) < bits_to_float(b); }

/* bubbleSort, oitCompositeDefines.glsl:51-89 (swaps on >=) */
static void bubble_sort(rec3* a, int n) {
  for (int i = n - 2; i >= 0; --i)
    for (int j = 0; j <= i; ++j)
      if (depth_ge(a[j].g, a[j + 1].g)) { rec3 t = a[j + 1]; a[j + 1] = a[j]; a[j] = t; }
}

/* insertionSort, oitCompositeDefines.glsl:94-109 */
static void insertion_sort(rec3* a, int L, rec3 item) {
  for (int i = 0; i < L; ++i) {
    if (depth_lt(item.g, a[i].g)) {
      for (int j = L - 1; j > i; --j) a[j] = a[j - 1];
      a[i] = item;
      return;
    }
  }
}

/* insertionSortTail, oitCompositeDefines.glsl:116-139 */
static rec3 insertion_sort_tail(rec3* a, int L, rec3 item) {
  rec3 newlast = item;
  if (depth_lt(item.g, a[L - 1].g)) {
    for (int i = 0; i < L; ++i) {
      if (depth_lt(item.g, a[i].g)) {
        newlast = a[L - 1];
        for (int j = L - 1; j > i; --j) a[j] = a[j - 1];
        a[i] = item;
        break;
      }
    }
  }
  return newlast;
}

/* Premultiplied colour of a sorted entry: the packed RGBA8 record, or with
 * RGBA32F linked-list records the float colour of the node it names. */
static rgba_d entry_colour(const or_frame* f, uint32_t r) {
  if (f->p.record_fp32 && f->p.algorithm == OR_LINKEDLIST) {
    const uint32_t* n = f->abuf + (size_t)r * 8;
    rgba_d c = {bits_to_float(n[0]), bits_to_float(n[1]), bits_to_float(n[2]), bits_to_float(n[3])};
    return premult(c);
  }
  return premult(decode_packed(r));
}

static rgba_d blend_array(const or_frame* f, const rec3* arr, int n) {
  rgba_d sum = zero_rgba();
  if (f->coverage) {
    /* oitSimple.frag.glsl:142-159 */
    for (int s = 0; s < f->S; ++s) {
      rgba_d sc = zero_rgba();
      for (int i = 0; i < n; ++i)
        if (arr[i].b & (1u << s)) do_blend(&sc, entry_colour(f, arr[i].r));
      sum.r += sc.r; sum.g += sc.g; sum.b += sc.b; sum.a += sc.a;
    }
    sum.r /= f->S; sum.g /= f->S; sum.b /= f->S; sum.a /= f->S;
  } else {
    for (int i = 0; i < n; ++i) do_blend(&sum, entry_colour(f, arr[i].r));
  }
  return sum;
}

static rgba_d composite_element(or_frame* f, size_t pixel, int s) {
  const int L = f->L;
  rec3 arr[32];
  size_t e = (size_t)s * f->P + pixel;
  switch (f->p.algorithm) {
    case OR_SIMPLE: case OR_SPINLOCK: case OR_INTERLOCK: {
      /* oitSimple.frag.glsl:115-169 (Spinlock/Interlock composites are identical) */
      int n = (int)f->aux[e];
      if (n > L) n = L;
      for (int i = 0; i < n; ++i) {
        const uint32_t* r = rec_ptr(f, s, pixel, i);
        arr[i].r = r[0]; arr[i].g = r[1]; arr[i].b = f->rec_words == 4 ? r[2] : 0;
      }
      bubble_sort(arr, n);
      return blend_array(f, arr, n);
    }
    case OR_LINKEDLIST: {
      /* oitLinkedList.frag.glsl:106-172 */
      /* RGBA32F nodes: the arrays carry node indices instead of colours */
      const int fp32 = f->p.record_fp32;
      int n = 0;
      uint32_t off = f->aux[e];
      while (off != 0 && n < L) {
        if (fp32) {
          const uint32_t* nd = f->abuf + (size_t)off * 8;
          arr[n].r = off; arr[n].g = nd[4]; arr[n].b = nd[5];
          off = nd[6];
        } else {
          const uint32_t* nd = f->abuf + (size_t)off * 4;
          arr[n].r = nd[0]; arr[n].g = nd[1]; arr[n].b = nd[2];
          off = nd[3];
        }
        n++;
      }
      bubble_sort(arr, n);
      rgba_d tail = zero_rgba();
      while (off != 0) {
        rec3 item;
        uint32_t next;
        if (fp32) {
          const uint32_t* nd = f->abuf + (size_t)off * 8;
          item.r = off; item.g = nd[4]; item.b = nd[5]; next = nd[6];
        } else {
          const uint32_t* nd = f->abuf + (size_t)off * 4;
          item.r = nd[0]; item.g = nd[1]; item.b = nd[2]; next = nd[3];
        }
        if (f->p.tail_blend) {
          rec3 t = insertion_sort_tail(arr, L, item);
          do_blend(&tail, entry_colour(f, t.r));
        } else {
          insertion_sort(arr, L, item);
        }
        off = next;
      }
      rgba_d sum = blend_array(f, arr, n);
      do_blend(&sum, tail);
      return sum;
    }
    case OR_LOOP: {
      /* oitLoop.frag.glsl:191-222 */
      size_t listPos = (size_t)s * 2 * L * f->P + pixel;
      int n = 0;
      for (int i = 0; i < L; ++i) {
        if (f->abuf[listPos + (size_t)i * f->P] != EMPTY32) n++; else break;
      }
      rgba_d sum = zero_rgba();
      for (int i = 0; i < n; ++i) do_blend_packed(&sum, f->abuf[listPos + (size_t)(L + i) * f->P]);
      return sum;
    }
    case OR_LOOP64: {
      /* oitLoop64.frag.glsl:162-183 */
      const uint64_t* ab = (const uint64_t*)f->abuf;
      const float* pay = f->p.record_fp32 ? (const float*)(f->abuf + f->E * (size_t)L * 2) : NULL;
      size_t listPos = (size_t)s * L * f->P + pixel;
      rgba_d sum = zero_rgba();
      for (int i = 0; i < L; ++i) {
        uint64_t k = ab[listPos + (size_t)i * f->P];
        if ((uint32_t)(k >> 32) == EMPTY32) break;
        if (pay) do_blend(&sum, premult_float(pay + 4 * (listPos + (size_t)i * f->P)));
        else do_blend_packed(&sum, (uint32_t)k);
      }
      return sum;
    }
    default: return zero_rgba();
  }
}

void or_composite(or_frame* f, uint8_t* out_rgba8, double* out_linear) {
  const int S = f->S;
  if (f->p.algorithm == OR_WEIGHTED) {
    /* oitWeighted.frag.glsl:98-108, blend main.cpp:578-588, per sample */
    OR_OMP("omp parallel for schedule(static)")
    for (size_t i = 0; i < (size_t)S * f->P; ++i) {
      rgba_d a = f->accum[i];
      or_real rv = f->reveal[i];
      or_real d = a.a > (or_real)1e-5 ? a.a : (or_real)1e-5;
      rgba_d* c = &f->color[i];
      c->r = (a.r / d) * (1.0 - rv) + c->r * rv;
      c->g = (a.g / d) * (1.0 - rv) + c->g * rv;
      c->b = (a.b / d) * (1.0 - rv) + c->b * rv;
      c->a = rv * (1.0 - rv) + c->a * rv;
    }
  } else {
    OR_OMP("omp parallel for schedule(dynamic, 1024)")
    for (size_t pixel = 0; pixel < f->P; ++pixel) {
      if (f->p.sample_shading) {
        for (int s = 0; s < S; ++s) {
          rgba_d sum = composite_element(f, pixel, s);
          rop_premultiplied(&f->color[(size_t)s * f->P + pixel], sum);
        }
      } else {
        rgba_d sum = composite_element(f, pixel, 0);
        for (int s = 0; s < S; ++s) rop_premultiplied(&f->color[(size_t)s * f->P + pixel], sum);
      }
    }
  }
  /* copyOffscreenToBackBuffer (main.cpp:645-774): MSAA resolve = box average
   * of samples; supersample = 2x2 box downsample; both in linear space. */
  const int ss = f->p.supersample > 1 ? f->p.supersample : 1;
  const int W = f->p.width, H = f->p.height;
  OR_OMP("omp parallel for schedule(static)")
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      rgba_d acc = zero_rgba();
      for (int dy = 0; dy < ss; ++dy)
        for (int dx = 0; dx < ss; ++dx) {
          size_t pixel = (size_t)(y * ss + dy) * f->RW + (size_t)(x * ss + dx);
          for (int s = 0; s < S; ++s) {
            rgba_d c = f->color[(size_t)s * f->P + pixel];
            acc.r += c.r; acc.g += c.g; acc.b += c.b; acc.a += c.a;
          }
        }
      or_real k = (or_real)1.0 / (or_real)(ss * ss * S);
      acc.r *= k; acc.g *= k; acc.b *= k; acc.a *= k;
      size_t o = (size_t)y * W + x;
      if (out_linear) {
        out_linear[4 * o + 0] = acc.r; out_linear[4 * o + 1] = acc.g;
        out_linear[4 * o + 2] = acc.b; out_linear[4 * o + 3] = acc.a;
      }
      if (out_rgba8) {
        out_rgba8[4 * o + 0] = (uint8_t)encode_double(acc.r);
        out_rgba8[4 * o + 1] = (uint8_t)encode_double(acc.g);
        out_rgba8[4 * o + 2] = (uint8_t)encode_double(acc.b);
        out_rgba8[4 * o + 3] = (uint8_t)unorm8_double(acc.a);
      }
    }
  }
}

void or_load_state(or_frame* f, const uint32_t* abuffer, const uint32_t* aux, const uint32_t* counter) {
  if (abuffer) memcpy(f->abuf, abuffer, f->abuf_words * 4);
  if (aux) memcpy(f->aux, aux, f->E * 4);
  if (counter) f->counter = *counter;
}

void or_load_color(or_frame* f, const double* rgba) {
  for (size_t i = 0; i < (size_t)f->S * f->P; ++i) {
    f->color[i].r = (or_real)rgba[4 * i + 0];
    f->color[i].g = (or_real)rgba[4 * i + 1];
    f->color[i].b = (or_real)rgba[4 * i + 2];
    f->color[i].a = (or_real)rgba[4 * i + 3];
  }
}

void or_set_ll_store_limit(or_frame* f, const uint32_t* limit) { f->ll_limit = limit; }

const void* or_buffer(const or_frame* f, int which, size_t* bytes) {
  size_t sp = (size_t)f->S * f->P;
  switch (which) {
    case OR_BUF_ABUFFER: if (bytes) *bytes = f->abuf_words * 4; return f->abuf;
    case OR_BUF_AUX: if (bytes) *bytes = f->E * 4; return f->aux;
    case OR_BUF_AUXDEPTH: if (bytes) *bytes = f->E * 4; return f->auxdepth;
    case OR_BUF_COUNTER: if (bytes) *bytes = 4; return &f->counter;
    case OR_BUF_DEPTH: if (bytes) *bytes = sp * 4; return f->depth;
    case OR_BUF_ACCUM: if (bytes) *bytes = sp * sizeof(rgba_d); return f->accum;
    case OR_BUF_REVEAL: if (bytes) *bytes = sp * sizeof(or_real); return f->reveal;
    case OR_BUF_COLOR: if (bytes) *bytes = sp * sizeof(rgba_d); return f->color;
    default: if (bytes) *bytes = 0; return NULL;
  }
}

uint64_t or_fragment_count(const or_frame* f) { return f->fragments; }
