/*
 * CPU oracle for the GB300 order-independent-transparency engine.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle the parity tests,
 * the smoke check and the bench's CPU-baseline leg compare the CUDA engine
 * against; no product code path loads or calls it.
 *
 * It is a single-threaded C restatement of the reference sample's transparent
 * pass (nvpro-samples/vk_order_independent_transparency): every fragment of
 * every triangle is produced by a software rasteriser (the fixed-point
 * raster specification below, which the CUDA rasteriser must reproduce bit
 * for bit) and pushed, in primitive order, through a line-by-line
 * restatement of the algorithm's COLOR/DEPTH fragment shader; the COMPOSITE
 * shader and the blend state are then evaluated per pixel in FP64.
 *
 * Parity status: the algorithm semantics are pinned by the known-answer
 * traces of the reference README (README.md:45, 53-66, 72, 80, 86-96), which
 * the CPU tests replay through or_inject_fragments(). The reference's mesh
 * generator (nvutils::createSphereUv), camera (nvutils::CameraManipulator) and
 * hardware rasteriser live outside the reference tree or in the GPU's fixed
 * function hardware, so mesh, camera and rasterisation parity is UNPINNED:
 * both sides consume the same mesh and matrices, and the rasteriser is this
 * project's own specification.
 */
#ifndef OIT_ORACLE_H
#define OIT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Algorithm ids: shaders/common.h:44-50. */
#define OR_SIMPLE 0
#define OR_LINKEDLIST 1
#define OR_LOOP 2
#define OR_LOOP64 3
#define OR_SPINLOCK 4
#define OR_INTERLOCK 5
#define OR_WEIGHTED 6

typedef struct or_params {
  int32_t algorithm;        /* OR_* */
  int32_t oit_layers;       /* OIT_LAYERS, 1..32 */
  int32_t nodes_per_pixel;  /* State::linkedListAllocatedPerElement (oit.h:68) */
  int32_t msaa;             /* 1, 4, 8 */
  int32_t sample_shading;   /* State::sampleShading */
  int32_t supersample;      /* 1 or 2; width/height below are the output size */
  int32_t tail_blend;       /* OIT_TAILBLEND */
  int32_t width, height;    /* output (viewport) size in pixels */
  float alpha_min, alpha_width; /* SceneData::alphaMin/alphaWidth (common.h:89-90) */
  int32_t record_fp32;      /* 1: RGBA32F records (linked list, Loop64): colours kept unquantised */
  float background[4];      /* render-pass clear colour, oitRender.cpp:90 */
} or_params;

typedef struct or_frame or_frame;

/* Spec helpers (also checked against the CUDA library's tables). */
float or_srgb_threshold(int k);       /* k in 0..254: smallest float encoding to >= k+1 */
double or_srgb_decode(int code);      /* sRGB8 code -> linear (double) */
uint32_t or_srgb_encode(float linear);/* linear float -> sRGB8 code */

or_frame* or_frame_create(const or_params* p);
void or_frame_destroy(or_frame* f);

/* Render-pass begin: colour = background, depth = 1.0 (oitRender.cpp:89-100). */
void or_begin(or_frame* f);
/* clearTransparent* (oitRender.cpp:156-356). */
void or_clear_transparent(or_frame* f);
/* Opaque draw (oitRender.cpp:113-122), back faces culled, depth LESS + write. */
void or_draw_opaque(or_frame* f, const float* proj_view, const float* view,
                    const float* vertices, const uint32_t* indices,
                    uint32_t first_triangle, uint32_t num_triangles);
/* COLOR (and Loop32 DEPTH) passes of drawTransparent* (oitRender.cpp:176-425). */
void or_draw_transparent(or_frame* f, const float* proj_view, const float* view,
                         const float* vertices, const uint32_t* indices,
                         uint32_t first_triangle, uint32_t num_triangles);
/* Inject n fragments in arrival order (the Loop32 DEPTH pass sees all of them
 * before its COLOR pass). xy: 2 ints per fragment; sample: per-fragment sample
 * index for sample shading (NULL = 0); rgba: linear unpremultiplied colour;
 * depth: window depth in [0,1]; mask: coverage mask (NULL = 1); view_z: view
 * space z for WBOIT (NULL = -1). Used by the known-answer tests. */
void or_inject_fragments(or_frame* f, int n, const int32_t* xy, const int32_t* sample,
                         const float* rgba, const float* depth, const uint32_t* mask,
                         const float* view_z);
/* COMPOSITE pass + blend onto the colour target + MSAA/SSAA resolve.
 * out_rgba8 (width*height*4, may be NULL), out_linear (width*height*4 doubles,
 * premultiplied linear, may be NULL). */
void or_composite(or_frame* f, uint8_t* out_rgba8, double* out_linear);

/* Replay: composite from A-buffer contents supplied by the caller (e.g. the
 * GPU's own linked-list pool), to check an order-dependent layout. The
 * buffers are copied into the frame before compositing. */
void or_load_state(or_frame* f, const uint32_t* abuffer, const uint32_t* aux,
                   const uint32_t* counter);

/* Replay: the colour target after tail blending (S*P premultiplied linear
 * RGBA doubles) supplied by the caller, e.g. a GPU frame whose tail blends ran
 * in arrival order. */
void or_load_color(or_frame* f, const double* rgba);

/* Per-pixel cap on stored linked-list nodes (replays the GPU's allocation
 * order on pool overflow); NULL disables. Array of render-size elements. */
void or_set_ll_store_limit(or_frame* f, const uint32_t* limit);

/* Accessors for parity checks. Buffer layouts equal the CUDA engine's. */
enum {
  OR_BUF_ABUFFER = 0,   /* u32 words */
  OR_BUF_AUX = 1,       /* u32 per element (count / list head) */
  OR_BUF_AUXDEPTH = 2,  /* u32 per element */
  OR_BUF_COUNTER = 3,   /* u32[1] */
  OR_BUF_DEPTH = 4,     /* u32 per sample (opaque depth buffer) */
  OR_BUF_ACCUM = 5,     /* double RGBA per sample (WBOIT) */
  OR_BUF_REVEAL = 6,    /* double per sample (WBOIT) */
  OR_BUF_COLOR = 7,     /* double RGBA per colour element after tail blend */
};
const void* or_buffer(const or_frame* f, int which, size_t* bytes);
uint64_t or_fragment_count(const or_frame* f);

/* The CPU legs' workload (oit_workload.c): the engine's seeded sphere scene
 * generator and camera, restated. Return 0, or -1 on invalid arguments.
 * Vertices: 10 floats each (pos.xyz, normal.xyz, color.rgba). */
int or_scene_size(uint32_t num_objects, uint32_t stacks, uint32_t slices, uint32_t* num_vertices,
                  uint32_t* num_triangles, uint32_t* triangles_per_object);
int or_scene_generate(uint64_t seed, uint32_t num_objects, uint32_t stacks, uint32_t slices, float half_extent,
                      float radius_min, float radius_max, float* vertices, uint32_t* indices);
int or_camera(uint32_t width, uint32_t height, const float eye[3], const float target[3], float fov_y_degrees,
              float z_near, float z_far, float* proj_view16, float* view16);

#ifdef __cplusplus
}
#endif
#endif
