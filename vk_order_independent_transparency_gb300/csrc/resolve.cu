// Batched resolve: the COMPOSITE pass of many views (linked list and Loop64,
// 1x, RGBA8 records) in one persistent launch.
//
//   k_rbin_count / k_rbin_scatter  counting sort of every view's 8x4
//                                  micro-tiles into cost buckets, costliest
//                                  bucket first. The cost of a micro-tile is
//                                  the most fragments any of its pixels
//                                  received (the transparent raster writes
//                                  it), i.e. the longest list its warp walks.
//   k_resolve_list / k_resolve_loop64  persistent: every warp resolves
//                                  micro-tiles (one lane per pixel) of one
//                                  view kind from the work list in a static
//                                  cyclic order.
//
// Per pixel the result equals the per-view composite (composite.cu, the same
// list walk, list_walk.cuh).
#include <type_traits>

#include "list_walk.cuh"
#include "oit_device.cuh"
#include "oit_internal.h"

namespace oit {
using namespace oitd;

namespace {

constexpr int kBinThreads = 256;
constexpr int kBinPerThread = 16;
constexpr int kBinChunk = kBinThreads * kBinPerThread;
constexpr uint32_t kEmptyKey = 0xFFFFFFFFu;

// the view holding global micro-tile g: the last view whose base is <= g
__device__ __forceinline__ int find_view(const uint32_t* tb, int n, uint32_t g) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tb[mid] <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Micro-tile (mx, my) of work item t of a view in the batch's order; false
// for the padding beyond the view's micro-tiles.
__device__ __forceinline__ bool item_microtile(const ResolveView& v, uint32_t t, int order, uint32_t& mx,
                                               uint32_t& my) {
  if (order == 0) {
    my = (uint32_t)(((uint64_t)t * v.ptx_recip) >> 40);
    mx = t - my * (uint32_t)v.ptx;
  } else {
    const uint32_t tile = t >> 3, sub = t & 7u;
    const uint32_t ty = (uint32_t)(((uint64_t)tile * v.tx_recip) >> 40);
    mx = 2u * (tile - ty * (uint32_t)v.tiles_x) + (sub & 1u);
    my = 4u * ty + (sub >> 1);
  }
  return mx < (uint32_t)v.mtx && my < (uint32_t)v.mty;
}

// Cost bucket of a micro-tile: 0 for no node reads, else 1 + floor(log2(cost))
// (edges 0) or the cost itself (edges 1), at most kResolveBuckets - 1. A list
// pixel reads one node per fragment; a Loop64 pixel reads its kept keys plus
// the terminating empty key.
__device__ __forceinline__ int tile_bucket(const ResolveView* __restrict__ views, const uint32_t* tb, int nv,
                                           uint32_t g, int order, int edges) {
  const int v = find_view(tb, nv, g);
  uint32_t mx, my;
  if (!item_microtile(views[v], g - tb[v], order, mx, my)) return 0;
  const uint32_t len = __ldg(views[v].lens + (size_t)my * views[v].mtx + mx);
  const int L = views[v].L;
  const uint32_t cost = views[v].kind == kResolveList ? len : min(len, (uint32_t)L) + (len < (uint32_t)L ? 1u : 0u);
  if (cost == 0) return 0;
  return edges ? (int)min(cost, (uint32_t)kResolveBuckets - 1u) : min(32 - __clz(cost), kResolveBuckets - 1);
}

__device__ __forceinline__ void load_bases(const ResolveBatch& b, uint32_t* tb) {
  for (int i = threadIdx.x; i < b.num_views; i += blockDim.x) tb[i] = b.tile_base[i];
  __syncthreads();
}

__global__ void __launch_bounds__(kBinThreads) k_rbin_count(ResolveBatch b) {
  __shared__ uint32_t tb[kResolveMaxViews];
  __shared__ uint32_t cnt[kResolveBuckets];
  if (threadIdx.x < kResolveBuckets) cnt[threadIdx.x] = 0;
  load_bases(b, tb);
  const uint32_t lane = threadIdx.x & 31;
  for (int i = 0; i < kBinPerThread; ++i) {
    const uint32_t g = blockIdx.x * kBinChunk + i * kBinThreads + threadIdx.x;
    const int bk = g < b.total_tiles ? tile_bucket(b.views, tb, b.num_views, g, b.order, b.edges) : -1;
    const uint32_t peers = __match_any_sync(0xffffffffu, bk);
    if (bk >= 0 && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&cnt[bk], (uint32_t)__popc(peers));
  }
  __syncthreads();
  if (threadIdx.x < kResolveBuckets && cnt[threadIdx.x]) atomicAdd(&b.hist[threadIdx.x], cnt[threadIdx.x]);
}

__global__ void __launch_bounds__(kBinThreads) k_rbin_scatter(ResolveBatch b) {
  __shared__ uint32_t tb[kResolveMaxViews];
  __shared__ uint32_t cnt[kResolveBuckets];
  __shared__ uint32_t base[kResolveBuckets];
  if (threadIdx.x < kResolveBuckets) cnt[threadIdx.x] = 0;
  load_bases(b, tb);
  const uint32_t lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
  int bk[kBinPerThread];
  uint32_t rank[kBinPerThread];
#pragma unroll
  for (int i = 0; i < kBinPerThread; ++i) {
    const uint32_t g = blockIdx.x * kBinChunk + i * kBinThreads + threadIdx.x;
    bk[i] = g < b.total_tiles ? tile_bucket(b.views, tb, b.num_views, g, b.order, b.edges) : -1;
    const uint32_t peers = __match_any_sync(0xffffffffu, bk[i]);
    const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
    uint32_t r = 0;
    if (bk[i] >= 0 && lane == leader) r = atomicAdd(&cnt[bk[i]], (uint32_t)__popc(peers));
    r = __shfl_sync(0xffffffffu, r, (int)leader);
    rank[i] = r + (uint32_t)__popc(peers & lt);
  }
  __syncthreads();
  if (threadIdx.x < kResolveBuckets) {
    // buckets are laid out costliest first
    uint32_t start = 0;
    for (int k = kResolveBuckets - 1; k > (int)threadIdx.x; --k) start += b.hist[k];
    base[threadIdx.x] = start + (cnt[threadIdx.x] ? atomicAdd(&b.fill[threadIdx.x], cnt[threadIdx.x]) : 0u);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < kBinPerThread; ++i) {
    const uint32_t g = blockIdx.x * kBinChunk + i * kBinThreads + threadIdx.x;
    if (bk[i] >= 0) b.items[base[bk[i]] + rank[i]] = g;
  }
}

// oitLoop64.frag.glsl:162-183: the keys are sorted; blend until the first
// empty one. key0 was fetched ahead; `nmax` bounds the keys to read (the
// micro-tile's longest list plus its terminator), fetched kLoop64Batch at a
// time without waiting on each other (lanes of a row share every layer's
// sectors).
constexpr int kLoop64Batch = 4;

__device__ __forceinline__ float4 resolve_loop64(const ResolveView& v, uint32_t pixel,
                                                 uint2 key0, int nmax) {
  const uint2* __restrict__ ab = reinterpret_cast<const uint2*>(v.abuf) + pixel;
  float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
  if (key0.y == kEmptyKey) return sum;
  blend_under(sum, decode_premult(key0.x));
  for (int i0 = 1; i0 < nmax; i0 += kLoop64Batch) {
    uint2 key[kLoop64Batch];
#pragma unroll
    for (int j = 0; j < kLoop64Batch; ++j)
      key[j] = i0 + j < nmax ? __ldg(ab + (size_t)(i0 + j) * v.P) : make_uint2(0u, kEmptyKey);
    bool done = false;
#pragma unroll
    for (int j = 0; j < kLoop64Batch; ++j) {
      done |= key[j].y == kEmptyKey;
      if (!done) blend_under(sum, decode_premult(key[j].x));
    }
    if (done) break;
  }
  return sum;
}

// The pixel of lane `lane` in work item `it`, or false outside the view. A
// warp's items only move forward through the views, so the view index `vi`
// (start at 0) is advanced instead of searched unless the list is binned.
struct ItemPixel {
  const ResolveView* v;
  uint32_t tile, pixel;
};

__device__ __forceinline__ bool item_pixel(const ResolveBatch& b, const uint32_t* tb, uint32_t it, int lane, int& vi,
                                           ItemPixel& o) {
  uint32_t g = it;
  if (b.items) {
    g = __ldg(b.items + it);
    vi = find_view(tb, b.num_views, g);
  } else {
    while (vi + 1 < b.num_views && tb[vi + 1] <= g) ++vi;
  }
  const ResolveView& v = b.views[vi];
  o.v = &v;
  uint32_t mx, my;
  if (!item_microtile(v, g - tb[vi], b.order, mx, my)) return false;
  o.tile = my * (uint32_t)v.mtx + mx;  // the micro-tile's index in the view's lengths
  const int x = (int)mx * 8 + (lane & 7), y = (int)my * 4 + (lane >> 3);
  if (x >= v.W || y >= v.H) return false;
  o.pixel = (uint32_t)y * (uint32_t)v.W + (uint32_t)x;
  return true;
}

// Persistent: every warp resolves micro-tiles (one lane per pixel) from the
// work list in static cyclic order. One kernel per view kind, so each gets the
// registers (and the occupancy) its own per-pixel work needs; the linked-list
// kernel keeps its sort arrays in local memory, or the first kSplitSlots
// entries in a shared-memory column (Split).
constexpr int kSplitSlots = 8;

// U micro-tiles per step: the independent first loads of all U (colour
// target, list head) are issued before any list is walked.
template <bool Split, int U, int Short = 0, int MinBlocks = 1>
__global__ void __launch_bounds__(256, MinBlocks) k_resolve_list(ResolveBatch b) {
  extern __shared__ __align__(16) uint32_t rsm[];
  load_bases(b, rsm);
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  using Arrays = typename std::conditional<Split, SplitArrays<kSplitSlots>, WalkArrays<false>>::type;
  Arrays a;
  uint32_t* col = rsm + ((b.num_views + 3) & ~3);
  if constexpr (Split) {
    a.sc = col + threadIdx.x;
    a.sd = col + kSplitSlots * blockDim.x + threadIdx.x;
    a.T = blockDim.x;
  }
  // Short: the thread's staging columns for short lists, [warp][Short][32]
  // colours then depths
  constexpr int kStage = Short > 0 ? Short : 1;
  uint32_t* stc = col + (threadIdx.x >> 5) * (2 * kStage * 32) + lane;
  uint32_t* std_ = stc + kStage * 32;
  int vi = 0;
  for (uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < b.total_tiles; it += U * warps) {
    ItemPixel ip[U];
    bool ok[U];
    float4 c[U];
    uint32_t head[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t iu = it + u * warps;
      ok[u] = iu < b.total_tiles && item_pixel(b, rsm, iu, lane, vi, ip[u]);
      if (ok[u]) {
        c[u] = load_color(ip[u].v->color, ip[u].v->color_half != 0, ip[u].pixel);
        head[u] = __ldg(ip[u].v->aux + ip[u].pixel);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (!ok[u]) continue;
      const ResolveView& v = *ip[u].v;
      const uint4* pool = reinterpret_cast<const uint4*>(v.abuf);
      float4 sum;
      // Short: a micro-tile whose longest list (the raster's count of the
      // fragments each pixel received, at least its list length) fits in 4
      // or Short entries and in OIT_LAYERS is staged and sorted by a network;
      // the choice is per warp
      bool done = false;
      if constexpr (Short > 0) {
        const int len = (int)__ldg(v.lens + ip[u].tile);
        if (len <= min(4, v.L))
          done = walk_list_staged<4>(pool, head[u], v.capacity, stc, std_, sum);
        else if (Short > 4 && len <= min(Short, v.L))
          done = walk_list_staged<Short>(pool, head[u], v.capacity, stc, std_, sum);
      }
      if (!done) sum = walk_list<false>(pool, head[u], v.capacity, v.L, v.tail, 1, a);
      rop_over(c[u], sum);
      write_rgba8(v.out, v.out_linear, ip[u].pixel, c[u]);
    }
  }
}

template <int U, int MinBlocks = 1>
__global__ void __launch_bounds__(256, MinBlocks) k_resolve_loop64(ResolveBatch b) {
  extern __shared__ __align__(16) uint32_t rsm[];
  load_bases(b, rsm);
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  int vi = 0;
  for (uint32_t it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < b.total_tiles; it += U * warps) {
    ItemPixel ip[U];
    bool ok[U];
    float4 c[U];
    uint2 key0[U];
    int nmax[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t iu = it + u * warps;
      ok[u] = iu < b.total_tiles && item_pixel(b, rsm, iu, lane, vi, ip[u]);
      if (ok[u]) {
        const ResolveView& v = *ip[u].v;
        c[u] = load_color(v.color, v.color_half != 0, ip[u].pixel);
        key0[u] = __ldg(reinterpret_cast<const uint2*>(v.abuf) + ip[u].pixel);
        nmax[u] = min((int)__ldg(v.lens + ip[u].tile) + 1, v.L);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (!ok[u]) continue;
      const ResolveView& v = *ip[u].v;
      const float4 sum = resolve_loop64(v, ip[u].pixel, key0[u], nmax[u]);
      rop_over(c[u], sum);
      write_rgba8(v.out, v.out_linear, ip[u].pixel, c[u]);
    }
  }
}

size_t resolve_smem(const ResolveBatch& b, int variant, int threads) {
  const size_t bases = (size_t)((b.num_views + 3) & ~3) * 4;
  const int slots = variant == kResolveVariantListShared || variant == kResolveVariantListShort8 ||
                            variant == kResolveVariantListShort8Dense
                        ? 8
                    : variant == kResolveVariantListShort4                                      ? 4
                                                                                                : 0;
  return bases + (size_t)threads * slots * 8;
}

template <class F>
cudaError_t with_kernel(int variant, F f) {
  switch (variant) {
    case kResolveVariantLoop64: return f(k_resolve_loop64<1>);
    case kResolveVariantLoop64x2: return f(k_resolve_loop64<2>);
    case kResolveVariantList: return f(k_resolve_list<false, 1>);
    case kResolveVariantListShared: return f(k_resolve_list<true, 1>);
    case kResolveVariantListx2: return f(k_resolve_list<false, 2>);
    case kResolveVariantListShort4: return f(k_resolve_list<false, 1, 4>);
    case kResolveVariantListShort8: return f(k_resolve_list<false, 1, 8>);
    case kResolveVariantListDense: return f(k_resolve_list<false, 1, 0, 8>);
    case kResolveVariantListShort8Dense: return f(k_resolve_list<false, 1, 8, 8>);
    case kResolveVariantLoop64Dense: return f(k_resolve_loop64<1, 8>);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t resolve_bin(const ResolveBatch& b, cudaStream_t s, uint64_t* launches) {
  if (!b.items || b.total_tiles == 0) return cudaSuccess;
  if (b.num_views > kResolveMaxViews) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(b.hist, 0, kResolveBuckets * sizeof(uint32_t), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.fill, 0, kResolveBuckets * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const uint32_t nb = (b.total_tiles + kBinChunk - 1) / kBinChunk;
  k_rbin_count<<<nb, kBinThreads, 0, s>>>(b);
  k_rbin_scatter<<<nb, kBinThreads, 0, s>>>(b);
  *launches += 2;
  return cudaGetLastError();
}

int resolve_blocks_per_sm(const ResolveBatch& b, int variant, int threads) {
  const size_t smem = resolve_smem(b, variant, threads);
  int n = 0;
  const cudaError_t e = with_kernel(variant, [&](auto kern) {
    if (smem > 48 * 1024) {
      const cudaError_t a = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (a != cudaSuccess) return a;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem);
  });
  return e == cudaSuccess ? n : 0;
}

cudaError_t resolve_run(const ResolveBatch& b, int variant, int threads, int blocks, cudaStream_t s) {
  if (b.total_tiles == 0) return cudaSuccess;
  if (b.num_views > kResolveMaxViews || threads % 32 != 0 || threads < 32 || threads > 256 || blocks < 1)
    return cudaErrorInvalidValue;
  return with_kernel(variant, [&](auto kern) {
    kern<<<blocks, threads, resolve_smem(b, variant, threads), s>>>(b);
    return cudaGetLastError();
  });
}

}  // namespace oit
