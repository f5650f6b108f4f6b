// Internal interface between the C++ host engine (engine.cpp) and the CUDA
// kernels (*.cu): parameter blocks and launch wrappers. Not part of the C ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace oit {

constexpr int kTile = 16;            // binning tile edge in pixels
constexpr int kWarpsPerTile = 8;     // one warp per 8x4 micro-tile
constexpr int kRasterWarpsPerBlock = 2;  // micro-tile warps per tile-raster CTA
// pair keys: tile id in the low 24 bits (sorted), the micro-tile mask above
constexpr int kMaskShift = 24;
constexpr uint32_t kTileKeyMask = (1u << kMaskShift) - 1u;
constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;

struct Mat4 {
  float m[16];
};

// Triangle setup: transform, cull, snap, bbox, interpolation constants.
struct SetupParams {
  const float* vertices;    // 10 floats per vertex; with instances: template vertices, 6 floats (pos, normal)
  const uint32_t* indices;  // 3 per triangle; with instances: the template's triangles
  const float* instances;   // null, or 8 floats per instance: centre.xyz, radius, color.rgba
  uint32_t template_triangles;  // triangles per instance
  uint32_t first_triangle;
  uint32_t num_triangles;
  // device memory: proj_view (16 floats, column-major) then view (16 floats),
  // 16-byte aligned. Read by the kernel, so a captured CUDA graph replays with
  // whatever the scene buffer holds when it runs (SceneData, shaders/common.h:77-92).
  const float* scene;
  int RW, RH;
  float alpha_min, alpha_width;
  uint32_t opaque_from;     // triangles t >= opaque_from (relative) are opaque: back faces culled, kind 0
  int samples;             // MSAA samples per pixel (1, 4, 8)
  int tiles_x;
  int num_tiles;           // key = tile + (transparent ? num_tiles : 0)
  // outputs
  // Per record, 2 * num_triangles of them: record t is triangle t, or the
  // first half of a triangle the near plane splits into two; its second half
  // is record num_triangles + t.
  uint2* bbox;            // pixel bbox (x0 | y0 << 16, x1 | y1 << 16); bit 31 of .y: a second half follows
  void* setup;            // TriSetup records (96 B)
  void* persp;            // TriPersp records (32 B, WBOIT only) or null
  uint32_t* pair_count;   // [num_triangles] tiles overlapped by both halves (0 = culled)
};

// The engine's view of a frame's geometry: a flattened triangle mesh
// (oit_mesh) or one template drawn per instance (oit_instanced_mesh).
struct MeshRef {
  const float* vertices;
  const uint32_t* indices;
  const float* instances;       // null for a flattened mesh
  uint32_t num_triangles;       // triangles of the frame
  uint32_t template_triangles;  // instanced: triangles per instance
};

// Tile bins of one draw: triangles sorted by tile, primitive order kept.
struct Bins {
  uint32_t* tile_begin;   // [num_tiles]
  uint32_t* tile_end;     // [num_tiles]
  uint32_t* tris;         // [capacity] triangle index per (tile, triangle) pair
  uint32_t* keys;         // [capacity] tile id per pair
  uint32_t* tris_alt;     // radix-sort ping-pong buffers
  uint32_t* keys_alt;
  uint32_t* pair_offset;  // [num_triangles + 1]
  uint32_t* scan_tmp;     // pair counts per 512-triangle block, scanned in place, then the scan's scratch
  uint32_t* hist;         // the radix sort's digit counts per chunk (and the scanned sort's scratch)
  uint32_t* total;        // [1] number of pairs (device)
  size_t capacity;
  // the radix sort keeps a view's pairs in at most 128 chunks up to this many
  // pairs (a view sorted beside others: they fill the GPU), and beyond it
  // spreads them over every block (a view sorted alone)
  size_t sort_direct_max;
};

enum class Alg : int {
  Simple = 0,
  LinkedList = 1,
  Loop = 2,
  Loop64 = 3,
  Spinlock = 4,
  Interlock = 5,
  Weighted = 6,
  Opaque = 7,
};

// Everything the tile rasteriser needs for one pass.
struct RasterParams {
  int RW, RH;
  int tiles_x, tiles_y;
  uint32_t P;                    // render pixels
  int S;                         // samples per pixel
  int ssn;                       // samples with their own A-buffer (sample shading), else 1
  int L;                         // OIT_LAYERS
  int tail;                      // OIT_TAILBLEND
  int coverage;                  // OIT_COVERAGE_SHADING
  const uint32_t* tile_begin;    // indexed by tile + tile_offset
  const uint32_t* tile_end;
  int tile_offset;               // 0: opaque lists, num_tiles: transparent lists
  const uint32_t* tile_tris;
  // the sorted pair keys beside tile_tris: tile id (bits 0-23) and the 8x4
  // micro-tiles of the tile that the triangle's bbox overlaps (bit 24 + k for
  // micro-tile k = 2 * row + column)
  const uint32_t* tile_keys;
  const uint2* bbox;
  const void* setup;
  const void* persp;
  // Bin overflow: when the draw's (tile, triangle) pairs exceed the bin
  // capacity, the pairs of the first triangles (triangle order) fill the bins
  // and the rest are dropped; the raster then walks its tile list for the
  // triangles that were binned whole and tests every later triangle of the
  // pass's range [pass_first, pass_end) by bbox. Null pair_total: no check.
  const uint32_t* pair_total;    // [1] the draw's pair count (device)
  const uint32_t* pair_offset;   // [num_tris] exclusive scan of pair_count
  const uint32_t* pair_count;    // [num_tris]
  uint32_t pair_capacity;
  uint32_t num_tris;             // triangles of the draw (bin-relative ids 0 .. num_tris - 1)
  uint32_t pass_first, pass_end; // this pass's triangles: transparent [0, opaque_from), opaque the rest
  // frame targets
  uint32_t* depth;               // [S][P] opaque depth (read by transparent passes)
  float4* opaque_color;          // [S][P]
  int has_opaque;                // 0: depth 1.0 and background colour everywhere
  float4 background;
  float4* color;                 // [ssn][P] colour target after tail blend (sample average unless sample shading)
  int color_half;                // the colour target holds four halves per element
  // algorithm state
  uint32_t* abuf;
  uint32_t* aux;
  uint32_t* auxdepth;
  uint32_t* counter;             // linked-list node counter
  uint32_t capacity;             // linked-list pool size in nodes
  int record_fp32;               // OIT_RECORD_RGBA32F
  void* accum;                   // WBOIT
  void* reveal;
  int weighted_fp32;
  uint32_t* error;
  unsigned long long* frag_count;
  // per 8x4 micro-tile: the most fragments any of its pixels received (capped
  // at 255), written by the transparent raster for the batched resolve's
  // work binning; null = not wanted (1x only)
  uint8_t* lens;
  int lens_stride;               // micro-tiles per row, (RW + 7) / 8
  // 1x transparent raster register budget: 32 runs the passes compiled for 36
  // resident warps per SM (56 registers) at 32 (64 registers); 0 = default
  int warps_per_sm;
};

// Several views' raster passes in one launch (the tile rasters of a batch):
// CTAs [cta_end[i-1], cta_end[i]) run view i's pass with v[i]. Passed as a
// kernel parameter (kMvMaxViews x RasterParams fits the parameter space).
constexpr int kMvMaxViews = 48;
struct MvRaster {
  int n;
  uint32_t cta_end[kMvMaxViews];
  RasterParams v[kMvMaxViews];
};

// The arrival-order linked-list COLOR pass (1x): triangles [0, num_tris) of
// the draw straight from their setup records, nodes linked by atomic head
// exchanges, pool overflow tail-blended under per-pixel locks.
struct ArrivalParams {
  int RW, RH;
  uint32_t P;
  uint32_t num_tris;
  uint32_t second_base;          // the draw's triangle count: record of the second half of a near-clipped t
  const uint2* bbox;
  const void* setup;
  const uint32_t* depth;         // [P] opaque depth
  const float4* opaque_color;    // [P]
  int has_opaque;
  float4 background;
  float4* color;                 // [P] colour target (initialised by the pass)
  int color_half;
  uint32_t* pool;                // uint4 nodes
  uint32_t* heads;               // [P]
  uint32_t* counter;
  uint32_t capacity;
  uint32_t* locks;               // [P] spin words (zeroed by the pass)
  int32_t held_lock;             // testing aid: this element's lock starts held (-1: none)
  int tail;
  uint32_t* error;
  unsigned long long* frag_count;
};

struct CompositeParams {
  int W, H;                      // output size
  int RW, RH;                    // render size
  int ss;                        // supersample factor
  uint32_t P;
  int S;
  int ssn;                       // samples with their own A-buffer (sample shading), else 1
  int L;
  int tail;
  int coverage;
  int record_fp32;
  int weighted_fp32;
  uint32_t capacity;             // linked-list pool size in nodes (walks are bounded by it)
  const uint32_t* abuf;
  const uint32_t* aux;
  const float4* color;           // [ssn][P] (A-buffer algorithms) colour after tail blend
  int color_half;                // four halves per element
  const float4* opaque_color;    // [S][P] (WBOIT) or null
  int has_opaque;
  float4 background;
  const void* accum;
  const void* reveal;
  uint8_t* out_rgba8;            // [W*H*4]
  float4* out_linear;            // optional [W*H]
};

// One view of the batched resolve (linked list or Loop64, 1x, RGBA8 records).
enum ResolveKind : int { kResolveList = 0, kResolveLoop64 = 1 };
struct ResolveView {
  const uint32_t* abuf;          // node pool (list) or keys [L][P] (Loop64)
  const uint32_t* aux;           // list heads [P]
  const float4* color;           // [P] colour target after tail blend
  uint8_t* out;                  // [P] RGBA8
  float4* out_linear;            // optional [P]
  const uint8_t* lens;           // [mty][mtx] per 8x4 micro-tile fragment counts
  uint32_t P, capacity;
  int W, H, L, kind, tail, mtx, mty;
  int color_half;
  // work items: the micro-tiles of the view's 16x16 tiles, 8 per tile, padded
  // to ptx = 2 * tiles_x columns; x / d = (x * recip) >> 40 with
  // recip = ceil(2^40 / d), exact for x < 2^26 and d <= 2^12
  int tiles_x, ptx;
  uint64_t tx_recip, ptx_recip;
  uint32_t tile_base;            // first global micro-tile index of this view
};

constexpr int kResolveBuckets = 8;
constexpr int kResolveMaxViews = 4096;

struct ResolveBatch {
  const ResolveView* views;      // [num_views] (device)
  const uint32_t* tile_base;     // [num_views] (device) copy of views[i].tile_base
  int num_views;
  uint32_t total_tiles;          // work items (micro-tiles, padded to whole tiles) over all views
  int order;                     // 0: micro-tiles row by row; 1: tile by tile (8 micro-tiles of a tile in a row)
  int edges;                     // cost buckets: 0 log2 (1, 2-3, 4-7, ...), 1 one per cost (1, 2, ..., 6, 7+)
  uint32_t* hist;                // [kResolveBuckets] (device)
  uint32_t* fill;                // [kResolveBuckets] (device)
  uint32_t* items;               // [total_tiles] work list, costliest bucket first; null = view order
};

// ---- launch wrappers (defined in the .cu files) -------------------------
cudaError_t bin_setup_scan(const SetupParams& sp, Bins& b, cudaStream_t s, uint64_t* launches);
cudaError_t bin_sort(const SetupParams& sp, Bins& b, int key_bits, int num_tiles, uint32_t* error, cudaStream_t s,
                     uint64_t* launches);
// with_scanned: room for the sort beyond sort_direct_max as well.
size_t radix_hist_words(size_t pairs, bool with_scanned);
// Triangle blocks of the clip and emit kernels, and the words of b.scan_tmp
// (their pair counts, scanned in place, and the scan's scratch).
size_t emit_blocks(size_t tris);
size_t bin_scan_words(size_t tris);
cudaError_t launch_raster_a(Alg alg, const RasterParams& p, cudaStream_t s);  // Simple, LinkedList, Opaque
cudaError_t launch_raster_b(Alg alg, const RasterParams& p, cudaStream_t s);  // Loop, Loop64
cudaError_t launch_raster_c(Alg alg, const RasterParams& p, cudaStream_t s);  // Spinlock, Interlock, Weighted
// Multi-view launches (every view of mv runs algorithm alg with one S / SSN);
// Alg::Opaque runs the views' opaque passes.
cudaError_t launch_raster_mv_a(Alg alg, const MvRaster& mv, cudaStream_t s);  // Simple, LinkedList, Opaque
cudaError_t launch_raster_mv_b(Alg alg, const MvRaster& mv, cudaStream_t s);  // Loop, Loop64
cudaError_t launch_raster_mv_c(Alg alg, const MvRaster& mv, cudaStream_t s);  // Spinlock, Interlock, Weighted
cudaError_t launch_composite(Alg alg, const CompositeParams& p, cudaStream_t s);
cudaError_t launch_arrival_ll(const ArrivalParams& p, cudaStream_t s, uint64_t* launches);  // arrival.cu
// Setup only (a draw whose rasters need no tile bins).
cudaError_t bin_setup_only(const SetupParams& sp, cudaStream_t s, uint64_t* launches);
// FP64 verification resolve (verify.cu): the composite recomputed in double;
// writes double4 linear colours to out_linear (may be null) and RGBA8 to
// p.out_rgba8 (may be null).
cudaError_t launch_composite_fp64(Alg alg, const CompositeParams& p, double* out_linear, cudaStream_t s);
// Batched resolve: bin the micro-tiles of every view by cost (costliest
// first), then one persistent launch resolves them all.
// Kernel variants: Loop64 views; linked-list views with their sort arrays in
// local memory, or with the first 8 entries in a shared-memory column; one or
// two micro-tiles per warp step.
enum ResolveVariant : int {
  kResolveVariantLoop64 = 0,
  kResolveVariantList = 1,
  kResolveVariantListShared = 2,
  kResolveVariantListx2 = 3,    // two micro-tiles per warp step
  kResolveVariantLoop64x2 = 4,  // two micro-tiles per warp step
  kResolveVariantListShort4 = 5,  // micro-tiles whose lists hold at most 4 (8) nodes staged in shared
  kResolveVariantListShort8 = 6,  // memory and sorted by a network; longer ones with the local arrays
  kResolveVariantListDense = 7,   // local arrays, at most 32 registers (eight 256-thread blocks per SM)
  kResolveVariantListShort8Dense = 8,  // Short8 at most 32 registers
  kResolveVariantLoop64Dense = 9,      // Loop64 at most 32 registers
};
cudaError_t resolve_bin(const ResolveBatch& b, cudaStream_t s, uint64_t* launches);
cudaError_t resolve_run(const ResolveBatch& b, int variant, int threads, int blocks, cudaStream_t s);
// Resident blocks per SM of a resolve variant for a block size (0 on error).
int resolve_blocks_per_sm(const ResolveBatch& b, int variant, int threads);
cudaError_t launch_fill_u32(uint32_t* dst, uint32_t value, size_t count, cudaStream_t s);
cudaError_t launch_fill_f4(float4* dst, float4 value, size_t count, cudaStream_t s);
size_t scan_scratch_words(size_t n);
void srgb_host_tables(float* thr256, float* dec256);

}  // namespace oit
