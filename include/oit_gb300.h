/*
 * oit_gb300.h - C ABI of the GB300-native order-independent-transparency engine.
 *
 * Drop-in for the transparent pass of nvpro-samples/vk_order_independent_transparency:
 * clearTransparent* -> drawTransparent* (COLOR/DEPTH + COMPOSITE) -> copy to the
 * back buffer, for the seven algorithms of the reference, on one GB300 (sm_103a).
 *
 * Conventions (all functions):
 *  - return an int status (OIT_OK or a negative OIT_ERR_*), never abort;
 *  - "stream" is a cudaStream_t passed as void* (NULL = legacy default stream);
 *    work is stream-ordered and asynchronous unless stated otherwise;
 *  - device buffers named *_device are CUDA device pointers owned by the caller;
 *    every other device buffer is owned by the context;
 *  - one context per host thread (the reference's Sample is single-threaded).
 */
#ifndef OIT_GB300_H
#define OIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Algorithms: shaders/common.h:44-50 (OIT_SIMPLE .. OIT_WEIGHTED). */
#define OIT_SIMPLE 0
#define OIT_LINKEDLIST 1
#define OIT_LOOP 2
#define OIT_LOOP64 3
#define OIT_SPINLOCK 4
#define OIT_INTERLOCK 5
#define OIT_WEIGHTED 6
#define OIT_NUM_ALGORITHMS 7

/* Antialiasing modes: shaders/common.h:58-64, expanded by
 * State::recomputeAntialiasingSettings (oit.h:84-115). */
#define OIT_AA_NONE 0
#define OIT_AA_MSAA_4X 1
#define OIT_AA_SSAA_4X 2
#define OIT_AA_SUPER_4X 3
#define OIT_AA_MSAA_8X 4
#define OIT_AA_SSAA_8X 5

/* Fragment record formats. RGBA8 is the reference's packed sRGB record
 * (packUnorm4x8, shaders/oitSimple.frag.glsl:70). RGBA32F is the plain FP32
 * record (unquantised linear colour), used as the precision/throughput
 * baseline; it is implemented for OIT_LINKEDLIST and OIT_LOOP64. */
#define OIT_RECORD_RGBA8 0
#define OIT_RECORD_RGBA32F 1

/* WBOIT accumulation precision: FP16 reproduces the reference's RGBA16F/R16F
 * targets (oit.h:234-235) by rounding after every blend; FP32 keeps float
 * accumulators. */
#define OIT_WEIGHTED_FP16 0
#define OIT_WEIGHTED_FP32 1

/* oit_state.flags */
#define OIT_FLAG_LINEAR_OUTPUT 0x1u  /* composite also writes OIT_BUF_OUTPUT_LINEAR */
#define OIT_FLAG_CUDA_GRAPH 0x2u     /* oit_render_frame replays a captured CUDA graph of the whole frame */
#define OIT_FLAG_HALF_COLOR 0x4u     /* colour target after tail blending stored as FP16 (blended in FP32
                                        within a tile, rounded once); the reference's is RGBA8 sRGB */
#define OIT_FLAG_ARRIVAL_ORDER 0x8u  /* linked list, 1x (and 2x2 supersampling), RGBA8 records: the COLOR pass
                                        as the reference's GPU runs it -- fragments of all triangles in
                                        parallel, nodes from the global counter linked by atomic exchanges
                                        of the head image in HBM (oitLinkedList.frag.glsl:51-85), pool
                                        overflow tail-blended under per-pixel spinlocks; list order is
                                        arrival order (not deterministic), the stored set per pixel is the
                                        same as in primitive order when the pool does not overflow. A frame
                                        without opaque objects needs no tile binning. Other states with it
                                        return OIT_ERR_UNSUPPORTED */

/* Status codes. */
#define OIT_OK 0
#define OIT_ERR_INVALID_ARGUMENT (-1)
#define OIT_ERR_UNSUPPORTED (-2)
#define OIT_ERR_OUT_OF_MEMORY (-3)
#define OIT_ERR_CUDA (-4)
#define OIT_ERR_DEVICE (-5)      /* a kernel raised a device error bit, see oit_get_error */
#define OIT_ERR_STATE (-6)       /* call made out of order (e.g. composite before draw) */
#define OIT_ERR_TOO_LARGE (-7)   /* the frame does not fit oit_render_frame_noalloc's scratch arena */

/* Device error bits reported by oit_get_error. */
#define OIT_DEVERR_BIN_OVERFLOW 0x1u  /* a draw's triangle/tile pairs exceeded the bin capacity sized on earlier
                                         frames: its image is still complete (the triangles that did not fit
                                         were tested by bbox, a slower walk) and the next frame call re-sizes
                                         the bins */
#define OIT_DEVERR_TIMEOUT 0x2u       /* a bounded wait gave up (an arrival-order tail blend's spinlock) */

/* Renderer settings: State (oit.h:64-116) plus the SceneData scalars
 * (shaders/common.h:77-92). */
typedef struct oit_state {
  uint32_t algorithm;                      /* OIT_SIMPLE .. OIT_WEIGHTED */
  uint32_t oit_layers;                     /* OIT_LAYERS: 1,2,4,8,16,32 */
  int32_t linked_list_allocated_per_element; /* A-buffer nodes per pixel/sample (LL) */
  int32_t tail_blend;                      /* OIT_TAILBLEND */
  int32_t interlock_is_ordered;            /* OIT_INTERLOCK_IS_ORDERED */
  uint32_t aa_type;                        /* OIT_AA_* */
  uint32_t width, height;                  /* viewport size in pixels */
  float alpha_min, alpha_width;            /* SceneData::alphaMin / alphaWidth */
  uint32_t record_format;                  /* OIT_RECORD_* */
  uint32_t weighted_precision;             /* OIT_WEIGHTED_* */
  float bin_capacity_scale;                /* tile-bin headroom over the (triangle, tile) pair count
                                              measured on earlier frames (0 = default 1.25) */
  uint32_t flags;                          /* OIT_FLAG_* */
} oit_state;

/* Per-frame scene constants: SceneData (shaders/common.h:77-92). Column-major
 * 4x4 matrices, vectors multiplied on the right (glm convention). */
typedef struct oit_scene_data {
  float proj_view_matrix[16];
  float view_matrix[16];
} oit_scene_data;

/* A triangle mesh in device memory. Vertex layout = the reference's Vertex
 * (utilities_vk.h:48-88): pos.xyz, normal.xyz, color.rgba, 40 bytes.
 * Indices: uint32 triangle list (main.cpp:340-386). */
typedef struct oit_mesh {
  const float* vertices_device;
  const uint32_t* indices_device;
  uint32_t num_vertices;
  uint32_t num_triangles;
} oit_mesh;

typedef struct oit_context oit_context;

/* Which context-owned buffer oit_get_buffer returns. */
#define OIT_BUF_ABUFFER 0        /* m_oitABuffer (oit.cpp:155-163) */
#define OIT_BUF_AUX 1            /* m_oitAuxImage: counts or list heads */
#define OIT_BUF_AUXDEPTH 2       /* m_oitAuxDepthImage (Spinlock/Interlock) */
#define OIT_BUF_COUNTER 3        /* m_oitCounterImage (Linked List) */
#define OIT_BUF_DEPTH 4          /* opaque depth, u32 per sample */
#define OIT_BUF_OPAQUE_COLOR 5   /* opaque colour, float4 per sample */
#define OIT_BUF_COLOR 6          /* colour target after tail blending, float4 */
#define OIT_BUF_ACCUM 7          /* WBOIT accumulation, half4 or float4 per sample */
#define OIT_BUF_REVEAL 8         /* WBOIT revealage, half or float per sample */
#define OIT_BUF_OUTPUT 9         /* resolved RGBA8 output image (width*height*4) */
#define OIT_BUF_OUTPUT_LINEAR 10 /* resolved premultiplied linear float4 output */
#define OIT_BUF_MICROTILE_LENGTHS 11 /* u8 per 8x4 micro-tile: most fragments any of its pixels received
                                        (batched-resolve views: linked list or Loop64, 1x, RGBA8) */

/* ---- lifetime ---------------------------------------------------------- */

/* Validates the state, sizes and allocates every per-frame buffer.
 * Replaces Sample::createFrameImages (oit.cpp:45-220) and the rebuild logic of
 * Sample::updateRendererFromState (main.cpp:130-250). */
int oit_create(const oit_state* state, oit_context** out_ctx);

/* Frees the context. Replaces Sample::onDetach / destroyFrameImages (oit.cpp:30-43). */
int oit_destroy(oit_context* ctx);

/* Sets the per-frame constants. Replaces Sample::updateUniformBuffer
 * (main.cpp:625-643), which records the upload into the frame's command
 * buffer: here the next frame call (oit_render_frame*, oit_draw_*,
 * oit_batch_render) copies them into the context's device scene buffer on
 * its own stream before its first kernel, so frames already queued keep the
 * constants they were called with and a replayed CUDA graph renders with the
 * newest ones. The host copy goes through a ring of 4 pinned slots: the call
 * blocks only when the copy made 4 updates ago has not run yet. */
int oit_update_scene(oit_context* ctx, const oit_scene_data* scene);

/* ---- per frame (the transparent pass) ---------------------------------- */

/* Clears the colour target to the background (0.2 linear) and depth to 1.0:
 * the main render pass begin (oitRender.cpp:89-100). */
int oit_begin_frame(oit_context* ctx, void* stream);

/* Clears the algorithm's auxiliary buffers. Replaces clearTransparentSimple /
 * LinkedList / Loop / Loop64 / Lock (oitRender.cpp:156-174, 201-216, 242-265,
 * 303-311, 337-356); WBOIT clears in its own pass (oitRender.cpp:394-397). */
int oit_clear_transparent(oit_context* ctx, void* stream);

/* Draws triangles [first_triangle, first_triangle + num_triangles) opaque
 * with depth test LESS and depth write, back faces culled.
 * Replaces the opaque vkCmdDrawIndexed of Sample::onRender (oitRender.cpp:113-122). */
int oit_draw_opaque(oit_context* ctx, const oit_mesh* mesh, uint32_t first_triangle,
                    uint32_t num_triangles, void* stream);

/* COLOR pass (and Loop32's DEPTH pass) of drawTransparent*: rasterises the
 * triangles, builds the algorithm's A-buffer and tail-blends overflow into the
 * colour target. Replaces the first draw(s) of drawTransparentSimple /
 * LinkedList / Loop / Loop64 / Lock / Weighted (oitRender.cpp:176-190, 218-230,
 * 267-291, 313-325, 358-371, 384-414). */
int oit_draw_transparent_color(oit_context* ctx, const oit_mesh* mesh, uint32_t first_triangle,
                               uint32_t num_triangles, void* stream);

/* COMPOSITE pass, fused with copyOffscreenToBackBuffer's MSAA resolve /
 * supersample downsample (main.cpp:645-774): writes width*height RGBA8 sRGB
 * pixels to out_rgba8_device (NULL = the context's OIT_BUF_OUTPUT).
 * Replaces the full-screen composite draws (oitRender.cpp:191-198, 232-239,
 * 293-300, 327-334, 373-381, 416-424). */
int oit_composite(oit_context* ctx, uint8_t* out_rgba8_device, void* stream);

/* FP64 verification resolve: the COMPOSITE pass of the context's current
 * frame (after oit_draw_transparent_color, oit_render_frame* or a batch)
 * recomputed in double precision from the same A-buffer, aux words and
 * tail-blended colour target -- the reference's sorts with doBlend /
 * doBlendPacked (shaders/shaderCommon.glsl:108-124) and the blend onto the
 * colour target (main.cpp:548-558) in FP64, then the MSAA / supersample
 * resolve. Writes width*height premultiplied linear double4 colours to
 * out_linear_device and/or RGBA8 sRGB pixels to out_rgba8_device (either may
 * be NULL, not both). Verification of the FP32 resolve, not part of a frame: no
 * counterpart in the reference, whose composite runs in FP32 shaders. */
int oit_verify_composite_fp64(oit_context* ctx, double* out_linear_device, uint8_t* out_rgba8_device, void* stream);

/* drawTransparent*(cmd, numObjects) (oit.h:379-425): COLOR + COMPOSITE over the
 * first num_triangles triangles of the mesh. */
int oit_draw_transparent(oit_context* ctx, const oit_mesh* mesh, uint32_t num_triangles,
                         uint8_t* out_rgba8_device, void* stream);

/* One whole frame as Sample::onRender (oitRender.cpp:28-154): begin, clear,
 * opaque draw of the last (100 - percent_transparent)% of the objects,
 * transparent draw of the first percent_transparent% and composite. */
int oit_render_frame(oit_context* ctx, const oit_mesh* mesh, uint32_t triangles_per_object,
                     int32_t percent_transparent, uint8_t* out_rgba8_device, void* stream);

/* Same frame from host memory: copies the mesh in and the RGBA8 image out
 * inside the call (synchronous on the stream). Host pointers may be pinned. */
int oit_render_frame_host(oit_context* ctx, const float* vertices_host, uint32_t num_vertices,
                          const uint32_t* indices_host, uint32_t num_triangles,
                          uint32_t triangles_per_object, int32_t percent_transparent,
                          uint8_t* out_rgba8_host, void* stream);

/* ---- instanced meshes -------------------------------------------------- */

/* One template mesh drawn once per instance: what Sample::initScene
 * (main.cpp:343-387) flattens into one vertex/index buffer, kept as a template
 * sphere plus a 32-byte record per object (the comment at main.cpp:343-345
 * names instancing as the alternative). No counterpart in the reference's
 * API. Template vertex: pos.xyz, normal.xyz (24 bytes). Instance: centre.xyz,
 * radius, color.rgba (32 bytes; the table must be 16-byte aligned). Frame
 * triangle t is template triangle t % template_triangles of instance
 * t / template_triangles; its positions are template_pos * radius + centre,
 * multiply and add each rounded to FP32, and its colour is the instance's, so
 * a frame is bit-identical to the frame of the flattened mesh that
 * oit_scene_generate builds from the same oit_scene_desc. */
typedef struct oit_instanced_mesh {
  const float* template_vertices_device;
  const uint32_t* template_indices_device;
  const float* instances_device;
  uint32_t template_vertices;
  uint32_t template_triangles;
  uint32_t num_instances;
} oit_instanced_mesh;

/* oit_render_frame over an instanced mesh: one object per instance, the first
 * percent_transparent% transparent. */
int oit_render_frame_instanced(oit_context* ctx, const oit_instanced_mesh* mesh, int32_t percent_transparent,
                               uint8_t* out_rgba8_device, void* stream);

/* Same frame from host memory (template, instance table in; RGBA8 image out),
 * synchronous on the stream. */
int oit_render_frame_instanced_host(oit_context* ctx, const float* template_vertices_host,
                                    uint32_t template_vertices, const uint32_t* template_indices_host,
                                    uint32_t template_triangles, const float* instances_host,
                                    uint32_t num_instances, int32_t percent_transparent,
                                    uint8_t* out_rgba8_host, void* stream);

/* One whole frame, like oit_render_frame, that allocates no device memory.
 * No counterpart in the reference: it exists for callers that cannot let a
 * library call cudaMalloc -- applications that own every device allocation
 * and give plugins a fixed budget, per-frame paths where cudaMalloc/cudaFree
 * may synchronise the device and stall other streams, and processes near a
 * device-memory limit where a mid-frame allocation can fail.
 * All per-frame scratch (setup records, tile bins, sort scratch, A-buffer,
 * colour and depth targets, the scene constants) lives in one 64 MiB device
 * array that every device loading the library holds until the process exits;
 * frames that do not fit return OIT_ERR_TOO_LARGE. The caller passes the
 * state, scene (host memory), mesh (device) and width*height*4 bytes of
 * device output. 1x and MSAA modes with RGBA8 records only (supersampling and
 * sample shading return OIT_ERR_UNSUPPORTED). Flags: OIT_FLAG_HALF_COLOR is
 * honoured (the image equals oit_render_frame's with the same flag),
 * OIT_FLAG_LINEAR_OUTPUT returns OIT_ERR_UNSUPPORTED (no linear image is
 * passed in) and OIT_FLAG_CUDA_GRAPH is ignored. The call is synchronous on
 * `stream`. The first call on a device looks up the array's device address
 * (once per device, with that device current; concurrent first calls on
 * several host threads each look it up and store the same value); make it
 * before any stream capture, and do not use the entry point across a
 * cudaDeviceReset (the address is not looked up again). Every call reuses the
 * same array, so calls that overlap on the GPU (other host threads, other
 * streams) race and must be serialised by the caller. */
int oit_render_frame_noalloc(const oit_state* state, const oit_scene_data* scene, const oit_mesh* mesh,
                             uint32_t triangles_per_object, int32_t percent_transparent,
                             uint8_t* out_rgba8_device, void* stream);

/* ---- batched views ----------------------------------------------------- */

/* One view of a batch: a context (own resolution, algorithm, OIT_LAYERS, record
 * format), its mesh and the frame parameters of oit_render_frame. A view with
 * an instanced mesh sets instanced_mesh (and leaves mesh NULL); its objects
 * are its instances and triangles_per_object is ignored. */
typedef struct oit_view_frame {
  oit_context* ctx;
  const oit_mesh* mesh;
  uint32_t triangles_per_object;
  int32_t percent_transparent;
  uint8_t* out_rgba8_device;  /* NULL = the view context's OIT_BUF_OUTPUT */
  const oit_instanced_mesh* instanced_mesh;
} oit_view_frame;

typedef struct oit_batch oit_batch;

/* A batch renders many views' frames as one CUDA graph in which the views run
 * concurrently on `parallel_streams` forked streams (0 = 8). The scene
 * constants of each view come from its context (oit_update_scene). */
int oit_batch_create(uint32_t parallel_streams, oit_batch** out_batch);
int oit_batch_destroy(oit_batch* batch);

/* Renders every view (Sample::onRender per view). The first call with a given
 * set of views renders them one by one (sizing their buffers) and captures the
 * graph; later calls replay it. Ordered after prior work on `stream`. */
int oit_batch_render(oit_batch* batch, const oit_view_frame* views, uint32_t num_views, void* stream);

/* Kernel launches per replay of the batch's graph. */
int oit_batch_launch_count(oit_batch* batch, uint64_t* launches);

/* COMPOSITE of every view's current frame (the composite draws of
 * drawTransparent*, oitRender.cpp:191-198 and 327-334, once per view in the
 * reference), for views whose frame has been rendered. Linked-list and Loop64
 * views at 1x with RGBA8 records and no linear output are resolved together:
 * one persistent launch for all linked-list views and one for all Loop64
 * views, running side by side; each walks the views' 8x4 micro-tiles, binned
 * by the longest per-pixel list of each (the transparent raster records it),
 * costliest first, or in view order. The other views get their own composite
 * launch. oit_batch_render resolves the same way. The first call for a set of
 * views times candidate shapes on these frames (an autotuner; see
 * oit_batch_resolve_config) and keeps the fastest. */
int oit_batch_resolve(oit_batch* batch, const oit_view_frame* views, uint32_t num_views, void* stream);

/* Tile rasters of a batch's graph. */
typedef struct oit_raster_config {
  int32_t multi_view;     /* 0: one raster launch per view and pass (views on the forked streams);
                             1: after every view's binning, one launch per pass, algorithm and sample
                             layout runs the CTAs of all its views, largest views first */
  uint32_t warps_per_sm;  /* register budget of the 1x linked-list, Simple, Loop64 and lock rasters:
                             36 resident warps per SM (56 registers, the default) or 32 (64 registers;
                             per-view launches only) */
  int32_t lane_order;     /* how views are spread over the forked streams: 0 round-robin in view order;
                             1 longest first: views in decreasing order of their frame time measured on
                             the batch's first (one by one) frames, each to the stream with the least
                             work so far */
} oit_raster_config;

/* Pins the batch's raster configuration; NULL (the default) lets the
 * autotuner capture the candidates (per-view launches at 36 and 32 warps per
 * SM, each with both lane orders, and multi-view launches) when the graph is
 * built, time them on the batch's own frames and keep the fastest. The next
 * oit_batch_render captures again. Unknown values return
 * OIT_ERR_INVALID_ARGUMENT. */
int oit_batch_set_raster_config(oit_batch* batch, const oit_raster_config* config);

/* The raster configuration of the batch's current graph; OIT_ERR_STATE
 * before the first capture. */
int oit_batch_raster_config(oit_batch* batch, oit_raster_config* config);

/* The shape the autotuner picked for one part of the batched resolve. */
typedef struct oit_resolve_shape {
  uint32_t threads_per_block;
  uint32_t blocks;          /* launched (with both parts present: this part's share of the machine) */
  int32_t binned;           /* 1: micro-tiles binned by list length, costliest first; 0: in order */
  int32_t tile_order;       /* 0: micro-tiles row by row; 1: the 8 micro-tiles of each 16x16 tile together */
  int32_t shared_slots;     /* sort-array entries per thread in shared memory (0 or 8; the rest local) */
  int32_t items_per_step;   /* micro-tiles a warp takes per step (1 or 2) */
  int32_t register_slots;   /* micro-tiles whose lists hold at most this many nodes (0, 4 or 8) are staged
                               in shared memory and sorted by a network in registers */
  int32_t dense;            /* 1: at most 32 registers per thread (eight 256-thread blocks per SM) */
  int32_t bin_edges;        /* binned work lists: 0 cost buckets 1, 2-3, 4-7, ... (log2); 1 one bucket per
                               cost 1, 2, ..., 6 and 7 or more */
} oit_resolve_shape;

/* Part 0: linked-list views, 1: Loop64 views. A part without views reports
 * zeros. OIT_ERR_STATE before the first resolve. */
int oit_batch_resolve_config(oit_batch* batch, uint32_t part, oit_resolve_shape* shape);

/* Pins the shape of one part of the batched resolve (a shape reported by
 * oit_batch_resolve_config, e.g. tuned once offline): the autotuner then
 * skips that part. blocks 0: every block that fits on the GPU. Shapes the
 * engine has no kernel for (for Loop64: shared or register slots; for linked
 * lists: more than one of shared slots, register slots and two items per
 * step, or dense with shared slots, register slots 4 or two items per step)
 * return OIT_ERR_INVALID_ARGUMENT. NULL unpins. The next render or resolve
 * of the batch uses it. */
int oit_batch_set_resolve_config(oit_batch* batch, uint32_t part, const oit_resolve_shape* shape);

/* ---- inspection -------------------------------------------------------- */

/* Testing aid for the error paths: the device allocation `after` allocations
 * from now (0: the next one) fails once with OIT_ERR_OUT_OF_MEMORY, as an
 * exhausted device would; -1 disarms it. Process-wide. The call that meets
 * the failure returns the error and leaves the context usable. */
int oit_debug_fail_allocations(int32_t after);

/* Testing aid for bounded waits: the context's next arrival-order frames
 * (OIT_FLAG_ARRIVAL_ORDER) start with the tail-blend lock of colour-target
 * element `element` already held, so a fragment that must tail-blend there
 * gives up after its bounded spin, is not blended, and the frame raises
 * OIT_DEVERR_TIMEOUT; the rest of the frame is unaffected. -1 releases it.
 * OIT_ERR_INVALID_ARGUMENT for an element outside the colour target. */
int oit_debug_hold_arrival_lock(oit_context* ctx, int32_t element);

/* Synchronises the context's last stream and returns the device error bits
 * (OIT_DEVERR_*) accumulated since the last call, then clears them. */
int oit_get_error(oit_context* ctx, uint32_t* device_error_bits);

/* Device pointer and size of a context-owned buffer (OIT_BUF_*). */
int oit_get_buffer(oit_context* ctx, int which, void** device_ptr, size_t* bytes);

/* Number of transparent fragments (after early depth) of the last COLOR pass;
 * synchronises the stream. */
int oit_get_fragment_count(oit_context* ctx, uint64_t* fragments);

/* Number of kernels the context launched since creation. */
int oit_get_launch_count(oit_context* ctx, uint64_t* launches);

/* Per-pass GPU timing with CUDA events recorded on the launching stream: the
 * role of nvvk::ProfilerGpuTimer::cmdFrameSection (oitRender.cpp:32, 82, 115,
 * 158, 182, 194, ...). Sections: */
#define OIT_PROF_OPAQUE_BIN 0        /* opaque setup + binning */
#define OIT_PROF_OPAQUE_RASTER 1     /* opaque tile raster */
#define OIT_PROF_TRANSPARENT_BIN 2   /* transparent setup + binning */
#define OIT_PROF_TRANSPARENT_RASTER 3/* COLOR (+DEPTH) tile raster: A-buffer build */
#define OIT_PROF_COMPOSITE 4         /* COMPOSITE + resolve */
#define OIT_PROF_NUM_SECTIONS 5

/* Enables (1) or disables (0) section timing; enabling resets the totals. */
int oit_profile_enable(oit_context* ctx, int enable);

/* Synchronises and returns, per section, the summed milliseconds and the
 * number of timed executions since profiling was enabled. */
int oit_profile_read(oit_context* ctx, double total_ms[OIT_PROF_NUM_SECTIONS],
                     uint64_t count[OIT_PROF_NUM_SECTIONS]);

/* Human-readable status. */
const char* oit_status_string(int status);

/* ---- host helpers (no GPU needed) -------------------------------------- */

/* Bytes of the A-buffer and auxiliary buffers for a state: the sizing rules of
 * Sample::createFrameImages (oit.cpp:100-201). */
int oit_abuffer_bytes(const oit_state* state, uint64_t* abuffer_bytes, uint64_t* aux_bytes);

/* Seeded synthetic sphere scene (the engine's stand-in for Sample::initScene,
 * main.cpp:334-417): num_objects UV spheres of `stacks` x `slices`, centres
 * uniform in [-half_extent, half_extent]^3, radii uniform in [radius_min,
 * radius_max], colour RGB uniform [0,1] and colour.a uniform [0,1] (mapped to
 * alpha by alpha_min/alpha_width), flattened into one mesh. */
typedef struct oit_scene_desc {
  uint64_t seed;
  uint32_t num_objects;
  uint32_t stacks, slices;
  float half_extent;
  float radius_min, radius_max;
} oit_scene_desc;

/* Sizes of the generated mesh. */
int oit_scene_size(const oit_scene_desc* desc, uint32_t* num_vertices, uint32_t* num_triangles,
                   uint32_t* triangles_per_object);

/* Fills host arrays of num_vertices*10 floats and num_triangles*3 indices. */
int oit_scene_generate(const oit_scene_desc* desc, float* vertices_host, uint32_t* indices_host);

/* The same scene as a template sphere and an instance table (see
 * oit_instanced_mesh): (stacks+1)*(slices+1) template vertices of 6 floats,
 * triangles_per_object*3 template indices, num_objects*8 instance floats. */
int oit_scene_generate_instanced(const oit_scene_desc* desc, float* template_vertices_host,
                                 uint32_t* template_indices_host, float* instances_host);

/* Camera at `eye` looking at `target` (up +y), vertical fov in degrees,
 * Vulkan clip space (z in [0,1], y down): the engine's stand-in for
 * CameraManipulator::getPerspectiveMatrix/getViewMatrix (main.cpp:630-631). */
int oit_camera(uint32_t width, uint32_t height, const float eye[3], const float target[3],
               float fov_y_degrees, float z_near, float z_far, oit_scene_data* out);

/* The engine's sRGB quantisation tables: 256 thresholds and 256 decoded
 * linear values (see gen_srgb_tables.py). */
int oit_srgb_tables(float* thresholds256, float* decode256);

/* ABI version (major*10000 + minor*100 + patch). */
int oit_version(void);

#ifdef __cplusplus
}
#endif
#endif
