// Allocation-free variant of oit_render_frame.
//
// Some callers cannot let a library call cudaMalloc: host applications that
// own every device allocation themselves and hand plugins a fixed memory
// budget (a renderer that sizes all its GPU memory at start-up), code on a
// latency-critical per-frame path where cudaMalloc/cudaFree may synchronise
// the whole device and stall other streams, and processes running close to a
// device-memory limit, where an allocation made in the middle of a frame can
// fail. oit_render_frame_noalloc serves them: every per-frame buffer the
// context path allocates (triangle setup records, tile bins, sort histograms
// and scan scratch, the A-buffer, the colour and depth targets) is carved out
// of one file-scope device array, reserved when the library is loaded. The
// caller passes only the inputs (state, scene, mesh) and the output image.
#include <atomic>
#include <cstdint>
#include <cstring>

#include "../../include/oit_gb300.h"
#include "oit_internal.h"

namespace {

// The scratch arena: 64 MiB on every device the library is loaded on, held
// until the process exits. Frames whose buffers do not fit are rejected with
// OIT_ERR_TOO_LARGE.
constexpr size_t kNoallocScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of the arena per device. In host code g_noalloc_scratch only
// names a host-side stand-in, so the address is looked up with
// cudaGetSymbolAddress, once per device, with that device current. Concurrent
// first calls may both look it up; they store the same value (atomically).
constexpr int kMaxDevices = 64;
std::atomic<unsigned char*> g_scratch_addr[kMaxDevices] = {};

cudaError_t scratch_base(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  unsigned char* a = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!a) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    a = static_cast<unsigned char*>(p);
    g_scratch_addr[dev].store(a, std::memory_order_release);
  }
  *out = a;
  return cudaSuccess;
}

struct Arena {
  unsigned char* base;
  size_t off, cap;
  template <class T>
  T* take(size_t bytes) {
    off = (off + 255) & ~(size_t)255;
    if (off + bytes > cap) return nullptr;
    T* p = reinterpret_cast<T*>(base + off);
    off += bytes;
    return p;
  }
};

bool layers_ok(uint32_t l) { return l == 1 || l == 2 || l == 4 || l == 8 || l == 16 || l == 32; }

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return OIT_OK;
  return e == cudaErrorMemoryAllocation ? OIT_ERR_OUT_OF_MEMORY : OIT_ERR_CUDA;
}

#define NOALLOC_TRY(expr)                         \
  do {                                            \
    cudaError_t _e = (expr);                      \
    if (_e != cudaSuccess) return status_of(_e);  \
  } while (0)

}  // namespace

extern "C" int oit_render_frame_noalloc(const oit_state* st, const oit_scene_data* scene, const oit_mesh* mesh,
                                        uint32_t tpo, int32_t percent, uint8_t* out_rgba8_device, void* stream) {
  using namespace oit;
  if (!st || !scene || !mesh || !out_rgba8_device || !tpo || percent < 0) return OIT_ERR_INVALID_ARGUMENT;
  if (!mesh->vertices_device || !mesh->indices_device || mesh->num_triangles < tpo) return OIT_ERR_INVALID_ARGUMENT;
  if (st->algorithm >= OIT_NUM_ALGORITHMS || !layers_ok(st->oit_layers) || st->width == 0 || st->height == 0 ||
      st->width > 16384 || st->height > 16384)
    return OIT_ERR_INVALID_ARGUMENT;
  if (st->algorithm == OIT_LINKEDLIST && st->linked_list_allocated_per_element < 1) return OIT_ERR_INVALID_ARGUMENT;
  int msaa = 1;
  switch (st->aa_type) {
    case OIT_AA_NONE: msaa = 1; break;
    case OIT_AA_MSAA_4X: msaa = 4; break;
    case OIT_AA_MSAA_8X: msaa = 8; break;
    case OIT_AA_SSAA_4X:
    case OIT_AA_SSAA_8X:
    case OIT_AA_SUPER_4X: return OIT_ERR_UNSUPPORTED;  // the arena path renders at the viewport size
    default: return OIT_ERR_INVALID_ARGUMENT;
  }
  if (st->record_format != OIT_RECORD_RGBA8) return OIT_ERR_UNSUPPORTED;
  // no linear output image is passed in; OIT_FLAG_CUDA_GRAPH does not apply
  // (the call is synchronous); OIT_FLAG_HALF_COLOR is honoured
  if (st->flags & OIT_FLAG_LINEAR_OUTPUT) return OIT_ERR_UNSUPPORTED;
  const bool half_color = (st->flags & OIT_FLAG_HALF_COLOR) != 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const Alg alg = static_cast<Alg>(st->algorithm);
  const int W = (int)st->width, H = (int)st->height, S = msaa, L = (int)st->oit_layers;
  const int coverage = msaa > 1;
  const uint64_t P = (uint64_t)W * (uint64_t)H;
  const int tiles_x = (W + kTile - 1) / kTile, tiles_y = (H + kTile - 1) / kTile;
  const int num_tiles = tiles_x * tiles_y;
  int key_bits = 1;
  while ((1 << key_bits) < 2 * num_tiles) ++key_bits;
  const uint32_t num_objects = mesh->num_triangles / tpo;
  uint32_t num_transparent = (uint32_t)(((uint64_t)num_objects * (uint32_t)percent) / 100u);
  if (num_transparent > num_objects) num_transparent = num_objects;
  const uint32_t N = num_objects * tpo, nt = num_transparent * tpo;
  const bool opaque = num_transparent < num_objects;
  const bool weighted = alg == Alg::Weighted;
  const bool wf32 = st->weighted_precision == OIT_WEIGHTED_FP32;
  const uint64_t capacity_nodes = alg == Alg::LinkedList ? (uint64_t)st->linked_list_allocated_per_element * P : 0;

  unsigned char* base = nullptr;
  NOALLOC_TRY(scratch_base(&base));
  Arena a{base, 0, kNoallocScratchBytes};
  uint32_t* words = a.take<uint32_t>(64);  // [0] error bits, [1] pair count, [2] node counter, [4..5] fragments
  float* scene_dev = a.take<float>(32 * sizeof(float));  // proj_view, view (read by the setup kernel)
  uint32_t* depth = opaque ? a.take<uint32_t>((size_t)S * P * 4) : nullptr;
  float4* opaque_color = opaque ? a.take<float4>((size_t)S * P * 16) : nullptr;
  float4* color = a.take<float4>((size_t)P * (half_color ? 8 : 16));
  size_t abuf_bytes = 0;
  switch (alg) {
    case Alg::Simple: case Alg::Spinlock: case Alg::Interlock: abuf_bytes = (size_t)P * L * (coverage ? 16 : 8); break;
    case Alg::LinkedList: abuf_bytes = (size_t)capacity_nodes * 16; break;
    case Alg::Loop: case Alg::Loop64: abuf_bytes = (size_t)P * L * 8; break;
    default: break;
  }
  uint32_t* abuf = abuf_bytes ? a.take<uint32_t>(abuf_bytes) : nullptr;
  uint32_t* aux = a.take<uint32_t>((size_t)P * 4);
  uint32_t* auxdepth = a.take<uint32_t>((size_t)P * 4);
  void* accum = weighted ? a.take<void>((size_t)S * P * (wf32 ? 16 : 8)) : nullptr;
  void* reveal = weighted ? a.take<void>((size_t)S * P * (wf32 ? 4 : 2)) : nullptr;
  // two records per triangle (the second half of a near-clipped one at N + t)
  void* setup = a.take<void>((size_t)N * 2 * 96);
  void* persp = weighted ? a.take<void>((size_t)N * 2 * 32) : nullptr;
  uint2* bbox = a.take<uint2>((size_t)N * 2 * 8);
  uint32_t* pair_count = a.take<uint32_t>((size_t)N * 4);
  uint32_t* pair_offset = a.take<uint32_t>(((size_t)N + 1) * 4);
  uint32_t* tile_begin = a.take<uint32_t>((size_t)2 * num_tiles * 4);
  uint32_t* tile_end = a.take<uint32_t>((size_t)2 * num_tiles * 4);
  if (!words || !scene_dev || (opaque && (!depth || !opaque_color)) || !color || (abuf_bytes && !abuf) || !aux ||
      !auxdepth || (weighted && (!accum || !reveal || !persp)) || !setup || !bbox || !pair_count || !pair_offset ||
      !tile_begin || !tile_end)
    return OIT_ERR_TOO_LARGE;
  // The rest holds the pairs (16 bytes each: keys, triangles, ping-pong), the
  // radix sort's digit counts and the pair-offset scan's words.
  const size_t left = a.cap - ((a.off + 255) & ~(size_t)255);
  const size_t reserve = (radix_hist_words(0, false) + bin_scan_words(N)) * 4 + 6 * 256;  // + alignment of 6 regions
  size_t pair_cap = left > reserve ? ((left - reserve) / 16) & ~(size_t)4095 : 0;
  const size_t hist_words = radix_hist_words(pair_cap, false);
  const size_t scan_n = bin_scan_words(N);
  Bins b{};
  b.keys = a.take<uint32_t>(pair_cap * 4);
  b.tris = a.take<uint32_t>(pair_cap * 4);
  b.keys_alt = a.take<uint32_t>(pair_cap * 4);
  b.tris_alt = a.take<uint32_t>(pair_cap * 4);
  b.hist = a.take<uint32_t>(hist_words * 4);
  b.scan_tmp = a.take<uint32_t>(scan_n * 4);
  if (pair_cap < 4096 || !b.keys || !b.tris || !b.keys_alt || !b.tris_alt || !b.hist || !b.scan_tmp)
    return OIT_ERR_TOO_LARGE;
  b.tile_begin = tile_begin;
  b.tile_end = tile_end;
  b.pair_offset = pair_offset;
  b.total = words + 1;
  b.capacity = pair_cap;
  b.sort_direct_max = ~(size_t)0;  // the arena holds the chunked sort's counts only

  // Calls share the arena and find the previous call's contents: clear what
  // must start at zero (error bits, pair count, node counter, fragment count).
  NOALLOC_TRY(cudaMemsetAsync(words, 0, 64, s));
  float scene_words[32];
  std::memcpy(scene_words, scene->proj_view_matrix, 16 * sizeof(float));
  std::memcpy(scene_words + 16, scene->view_matrix, 16 * sizeof(float));
  NOALLOC_TRY(cudaMemcpyAsync(scene_dev, scene_words, sizeof(scene_words), cudaMemcpyHostToDevice, s));
  const float4 bg = make_float4(0.2f, 0.2f, 0.2f, 0.2f);  // oitRender.cpp:90
  if (opaque) {
    NOALLOC_TRY(launch_fill_u32(depth, 0x3F800000u, (size_t)S * P, s));
    NOALLOC_TRY(launch_fill_f4(opaque_color, bg, (size_t)S * P, s));
  }
  SetupParams sp{};
  sp.vertices = mesh->vertices_device;
  sp.indices = mesh->indices_device;
  sp.first_triangle = 0;
  sp.num_triangles = N;
  sp.scene = scene_dev;
  sp.RW = W;
  sp.RH = H;
  sp.alpha_min = st->alpha_min;
  sp.alpha_width = st->alpha_width;
  sp.opaque_from = nt;
  sp.samples = S;
  sp.tiles_x = tiles_x;
  sp.num_tiles = num_tiles;
  sp.bbox = bbox;
  sp.setup = setup;
  sp.persp = persp;
  sp.pair_count = pair_count;
  uint64_t launches = 0;
  NOALLOC_TRY(bin_setup_scan(sp, b, s, &launches));
  uint32_t pairs = 0;
  NOALLOC_TRY(cudaMemcpyAsync(&pairs, b.total, 4, cudaMemcpyDeviceToHost, s));
  NOALLOC_TRY(cudaStreamSynchronize(s));
  if (pairs > pair_cap) return OIT_ERR_TOO_LARGE;  // more (tile, triangle) pairs than the arena holds
  // the sort's grids and histogram scans follow the capacity: size it to this
  // frame's pairs (the regions carved for pair_cap cover the smaller one)
  b.capacity = ((size_t)pairs + 4095) & ~(size_t)4095;
  if (b.capacity < 4096) b.capacity = 4096;
  NOALLOC_TRY(bin_sort(sp, b, key_bits, num_tiles, words, s, &launches));

  RasterParams p{};
  p.RW = W;
  p.RH = H;
  p.tiles_x = tiles_x;
  p.tiles_y = tiles_y;
  p.P = (uint32_t)P;
  p.S = S;
  p.ssn = 1;
  p.L = L;
  p.tail = st->tail_blend ? 1 : 0;
  p.coverage = coverage;
  p.tile_begin = b.tile_begin;
  p.tile_end = b.tile_end;
  p.tile_tris = b.tris;
  p.tile_keys = b.keys;
  p.pair_total = b.total;
  p.pair_offset = pair_offset;
  p.pair_count = pair_count;
  p.pair_capacity = (uint32_t)b.capacity;
  p.num_tris = N;
  p.bbox = bbox;
  p.setup = setup;
  p.persp = persp;
  p.depth = depth;
  p.opaque_color = opaque_color;
  p.has_opaque = opaque ? 1 : 0;
  p.background = bg;
  p.color = color;
  p.color_half = half_color ? 1 : 0;
  p.abuf = abuf;
  p.aux = aux;
  p.auxdepth = auxdepth;
  p.counter = words + 2;
  p.capacity = (uint32_t)capacity_nodes;
  p.record_fp32 = 0;
  p.accum = accum;
  p.reveal = reveal;
  p.weighted_fp32 = wf32 ? 1 : 0;
  p.error = words;
  p.frag_count = reinterpret_cast<unsigned long long*>(words + 4);
  if (opaque) {
    p.tile_offset = 0;
    p.pass_first = nt;
    p.pass_end = N;
    NOALLOC_TRY(launch_raster_a(Alg::Opaque, p, s));
  }
  p.tile_offset = num_tiles;
  p.pass_first = 0;
  p.pass_end = nt;
  switch (alg) {
    case Alg::Simple: case Alg::LinkedList: NOALLOC_TRY(launch_raster_a(alg, p, s)); break;
    case Alg::Loop: case Alg::Loop64: NOALLOC_TRY(launch_raster_b(alg, p, s)); break;
    default: NOALLOC_TRY(launch_raster_c(alg, p, s)); break;
  }
  CompositeParams c{};
  c.W = W;
  c.H = H;
  c.RW = W;
  c.RH = H;
  c.ss = 1;
  c.P = (uint32_t)P;
  c.S = S;
  c.ssn = 1;
  c.L = L;
  c.tail = p.tail;
  c.coverage = coverage;
  c.record_fp32 = 0;
  c.weighted_fp32 = p.weighted_fp32;
  c.capacity = p.capacity;
  c.abuf = abuf;
  c.aux = aux;
  c.color = color;
  c.color_half = half_color ? 1 : 0;
  c.opaque_color = opaque_color;
  c.has_opaque = p.has_opaque;
  c.background = bg;
  c.accum = accum;
  c.reveal = reveal;
  c.out_rgba8 = out_rgba8_device;
  c.out_linear = nullptr;
  NOALLOC_TRY(launch_composite(alg, c, s));
  uint32_t err = 0;
  NOALLOC_TRY(cudaMemcpyAsync(&err, words, 4, cudaMemcpyDeviceToHost, s));
  NOALLOC_TRY(cudaStreamSynchronize(s));
  return err ? OIT_ERR_DEVICE : OIT_OK;
}
