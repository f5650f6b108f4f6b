// Internal interface between the C++ host engine (engine.cpp) and the CUDA
// kernels (*.cu): parameter blocks and launch wrappers. Not part of the C ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace oit {

constexpr int kTile = 16;            // binning tile edge in pixels
constexpr int kWarpsPerTile = 8;     // one warp per 8x4 micro-tile
constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;

struct Mat4 {
  float m[16];
};

// Triangle setup: transform, cull, snap, bbox, interpolation constants.
struct SetupParams {
  const float* vertices;
  const uint32_t* indices;
  uint32_t first_triangle;
  uint32_t num_triangles;
  Mat4 proj_view;
  Mat4 view;
  int RW, RH;
  float alpha_min, alpha_width;
  uint32_t opaque_from;     // triangles t >= opaque_from (relative) are opaque: back faces culled, kind 0
  int samples;             // MSAA samples per pixel (1, 4, 8)
  int tiles_x;
  int num_tiles;           // key = tile + (transparent ? num_tiles : 0)
  // outputs
  uint2* bbox;            // [num_triangles] pixel bbox (x0 | y0 << 16, x1 | y1 << 16)
  void* setup;            // [num_triangles] TriSetup records (96 B)
  void* persp;            // [num_triangles] TriPersp records (32 B, WBOIT only) or null
  uint32_t* pair_count;   // [num_triangles] tiles overlapped (0 = culled)
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
  uint32_t* scan_tmp;     // scan scratch
  uint32_t* hist;         // radix histograms
  uint32_t* total;        // [1] number of pairs (device)
  size_t capacity;
  size_t scan_tmp_words;
  size_t hist_words;
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
  const uint2* bbox;
  const void* setup;
  const void* persp;
  // frame targets
  uint32_t* depth;               // [S][P] opaque depth (read by transparent passes)
  float4* opaque_color;          // [S][P]
  int has_opaque;                // 0: depth 1.0 and background colour everywhere
  float4 background;
  float4* color;                 // [ssn][P] colour target after tail blend (sample average unless sample shading)
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
  const float4* opaque_color;    // [S][P] (WBOIT) or null
  int has_opaque;
  float4 background;
  const void* accum;
  const void* reveal;
  uint8_t* out_rgba8;            // [W*H*4]
  float4* out_linear;            // optional [W*H]
};

// ---- launch wrappers (defined in the .cu files) -------------------------
cudaError_t bin_setup_scan(const SetupParams& sp, Bins& b, cudaStream_t s, uint64_t* launches);
cudaError_t bin_sort(const SetupParams& sp, Bins& b, int key_bits, int num_tiles, uint32_t* error, cudaStream_t s,
                     uint64_t* launches);
size_t radix_hist_words(size_t pairs);
cudaError_t launch_raster_a(Alg alg, const RasterParams& p, cudaStream_t s);  // Simple, LinkedList, Opaque
cudaError_t launch_raster_b(Alg alg, const RasterParams& p, cudaStream_t s);  // Loop, Loop64
cudaError_t launch_raster_c(Alg alg, const RasterParams& p, cudaStream_t s);  // Spinlock, Interlock, Weighted
cudaError_t launch_composite(Alg alg, const CompositeParams& p, cudaStream_t s);
cudaError_t launch_fill_u32(uint32_t* dst, uint32_t value, size_t count, cudaStream_t s);
cudaError_t launch_fill_f4(float4* dst, float4 value, size_t count, cudaStream_t s);
size_t scan_scratch_words(size_t n);
void srgb_host_tables(float* thr256, float* dec256);

}  // namespace oit
