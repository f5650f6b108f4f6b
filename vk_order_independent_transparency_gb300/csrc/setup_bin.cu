// Triangle setup and order-preserving tile binning.
//
// The reference hands its triangles to the fixed-function pipeline
// (vkCmdDrawIndexed in oitRender.cpp:185, 226, 275, 287, 321, 367, 413), which
// runs object.vert.glsl and rasterises them while keeping primitive order for
// blending. Here the same work is split into:
//   k_setup       one thread per triangle: transform, cull, snap to 1/256 px,
//                 bbox, interpolation constants (the raster specification);
//   k_setup_clip  the same for the triangles that cross the near plane,
//                 clipped into one or two; the pair count of every
//                 512-triangle block;
//   scan + emit   the blocks' pair counts scanned, then one (tile, triangle)
//                 pair per 16x16 tile the bbox touches, written in triangle
//                 order; the key holds the tile id (bits 0-23) and the 8x4
//                 micro-tiles the bbox overlaps (bits 24-31);
//   radix sort    stable LSD sort of the pairs by tile id, 8 bits a pass, in
//                 chunks (digit counts, then a scatter with warp-private
//                 ranks), so every tile's list keeps primitive order (the
//                 mask bits ride along unsorted);
//   k_tile_bounds begin/end of each tile's list (where the sorted tile id
//                 changes).
#include <algorithm>
#include <cstdio>

#include "oit_device.cuh"
#include "oit_internal.h"

namespace oit {
using namespace oitd;

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096 elements per block
constexpr int kRadixThreads = 256;
constexpr int kRadixRounds = 8;
constexpr int kRadixBits = 8;
constexpr int kRadixBins = 1 << kRadixBits;

// ---------------------------------------------------------------------------
// Setup (object.vert.glsl:32-39 + near-plane clip + viewport transform +
// triangle setup)
// ---------------------------------------------------------------------------
// One clip-space vertex with the attributes the raster interpolates.
struct ClipVert {
  float x, y, z, w, vz, nx, ny, nz;
};

// The vertex where edge a -> b crosses the near plane z = 0 (Vulkan clip
// space): attributes interpolated linearly at t = za / (za - zb), z exactly 0.
__device__ __forceinline__ ClipVert near_cut(const ClipVert& a, const ClipVert& b) {
  const float t = __fdiv_rn(a.z, __fsub_rn(a.z, b.z));
  ClipVert r;
  r.x = __fmaf_rn(t, __fsub_rn(b.x, a.x), a.x);
  r.y = __fmaf_rn(t, __fsub_rn(b.y, a.y), a.y);
  r.z = 0.0f;
  r.w = __fmaf_rn(t, __fsub_rn(b.w, a.w), a.w);
  r.vz = __fmaf_rn(t, __fsub_rn(b.vz, a.vz), a.vz);
  r.nx = __fmaf_rn(t, __fsub_rn(b.nx, a.nx), a.nx);
  r.ny = __fmaf_rn(t, __fsub_rn(b.ny, a.ny), a.ny);
  r.nz = __fmaf_rn(t, __fsub_rn(b.nz, a.nz), a.nz);
  return r;
}

// Setup of one triangle of clip-space vertices into record `slot`: the
// 0 <= z <= w, w > 0 test, projection, snap, orientation (back faces culled
// for opaque triangles), bbox, the small-triangle sample test and the record.
// Writes bbox[slot] (empty when dropped, bit 31 of .y = has_second) and
// returns the number of tiles the bbox overlaps (0 when dropped).
__device__ __forceinline__ uint32_t setup_half(const SetupParams& p, int S, uint32_t slot, bool opaque,
                                               const ClipVert (&cv)[3], const float* c0, bool has_second) {
  const uint32_t second_bit = has_second ? 0x80000000u : 0u;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (!(cv[k].w > 0.0f) || !(cv[k].z >= 0.0f) || !(cv[k].z <= cv[k].w)) ok = false;
  int X[3], Y[3];
  float zz[3], q[3];
  if (ok) {
    const float halfW = 0.5f * (float)p.RW, halfH = 0.5f * (float)p.RH;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      q[k] = __fdiv_rn(1.0f, cv[k].w);
      const float ndx = __fmul_rn(cv[k].x, q[k]), ndy = __fmul_rn(cv[k].y, q[k]);
      zz[k] = __fmul_rn(cv[k].z, q[k]);
      const float sx = __fmaf_rn(ndx, halfW, halfW), sy = __fmaf_rn(ndy, halfH, halfH);
      if (!(fabsf(sx) < 16384.0f) || !(fabsf(sy) < 16384.0f)) ok = false;
      X[k] = __float2int_rn(__fmul_rn(sx, 256.0f));
      Y[k] = __float2int_rn(__fmul_rn(sy, 256.0f));
    }
  }
  long long area = 0;
  if (ok) {
    area = (long long)(X[1] - X[0]) * (long long)(Y[2] - Y[0]) - (long long)(Y[1] - Y[0]) * (long long)(X[2] - X[0]);
    if (area == 0) ok = false;
    // area > 0: clockwise on the y-down framebuffer = back face for
    // VK_FRONT_FACE_COUNTER_CLOCKWISE (main.cpp:520-525); only opaque
    // triangles cull back faces (transparent ones are double-sided, oit.cpp:703).
    if (area > 0 && opaque) ok = false;
  }
  // counter-clockwise (area < 0) triangles swap vertices 1 and 2 so that
  // every record winds one way; selects, not an index, keep it in registers
  const bool sw = ok && area < 0;
  if (sw) area = -area;
  int bx0 = 0, by0 = 0, bx1 = -1, by1 = -1;
  int PX[3], PY[3];
  if (ok) {
    PX[0] = X[0]; PY[0] = Y[0];
    PX[1] = sw ? X[2] : X[1]; PY[1] = sw ? Y[2] : Y[1];
    PX[2] = sw ? X[1] : X[2]; PY[2] = sw ? Y[1] : Y[2];
    const int minX = min(PX[0], min(PX[1], PX[2])), maxX = max(PX[0], max(PX[1], PX[2]));
    const int minY = min(PY[0], min(PY[1], PY[2])), maxY = max(PY[0], max(PY[1], PY[2]));
    bx0 = max(minX >> 8, 0);
    by0 = max(minY >> 8, 0);
    bx1 = min(maxX >> 8, p.RW - 1);
    by1 = min(maxY >> 8, p.RH - 1);
    if (bx0 > bx1 || by0 > by1) ok = false;
  }
  int tl = 0;
  if (ok) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int a = (i + 1) % 3, b = (i + 2) % 3;
      const int dx = PX[b] - PX[a], dy = PY[b] - PY[a];
      if (dy < 0 || (dy == 0 && dx > 0)) tl |= 1 << i;
    }
  }
  // Small triangles: test every sample of the (at most 2x2 pixel) bbox now,
  // so triangles that cover no sample never reach the bins.
  if (ok && (bx1 - bx0) <= 1 && (by1 - by0) <= 1) {
    const int4 a = make_int4(PX[0], PY[0], PX[1], PY[1]);
    const int4 b = make_int4(PX[2], PY[2], tl, 0);
    bool any = false;
    for (int py = by0; py <= by1; ++py)
      for (int px = bx0; px <= bx1; ++px)
        for (int s = 0; s < S; ++s) {
          int2 sp = S == 8 ? sample_pos<8>(s) : (S == 4 ? sample_pos<4>(s) : sample_pos<1>(s));
          if (inside(edges_at(a, b, px * 256 + sp.x, py * 256 + sp.y), tl)) any = true;
        }
    if (!any) ok = false;
  }
  if (!ok) {
    // an empty bbox (x0 > x1): the unbinned walk of an overflowed frame
    // tests every triangle's bbox
    p.bbox[slot] = make_uint2(0xFFFFFFFFu, second_bit);
    return 0;
  }
  TriSetup T;
  T.xy01 = make_int4(PX[0], PY[0], PX[1], PY[1]);
  float alpha = __fmaf_rn(__ldg(c0 + 3), p.alpha_width, p.alpha_min);
  alpha = (alpha > 0.0f) ? alpha : 0.0f;
  alpha = (alpha < 1.0f) ? alpha : 1.0f;
  const int acode = __float2int_rn(__fmul_rn(alpha, 255.0f));
  const int minX = min(PX[0], min(PX[1], PX[2])), maxX = max(PX[0], max(PX[1], PX[2]));
  const int minY = min(PY[0], min(PY[1], PY[2])), maxY = max(PY[0], max(PY[1], PY[2]));
  const int small = (maxX - minX < kSmallExtent && maxY - minY < kSmallExtent) ? kFlagSmall : 0;
  T.xy2f = make_int4(PX[2], PY[2], tl | small | (acode << 8), __float_as_int(alpha));
  const float z0 = zz[0], z1 = sw ? zz[2] : zz[1], z2 = sw ? zz[1] : zz[2];
  T.zc = make_float4(z0, __fsub_rn(z1, z0), __fsub_rn(z2, z0), __fdiv_rn(1.0f, __ll2float_rn(area)));
  const float q0 = q[0], q1 = sw ? q[2] : q[1], q2 = sw ? q[1] : q[2];
  const ClipVert& v1 = sw ? cv[2] : cv[1];
  const ClipVert& v2 = sw ? cv[1] : cv[2];
  T.n0 = make_float4(__fmul_rn(cv[0].nx, q0), __fmul_rn(cv[0].ny, q0), __fmul_rn(cv[0].nz, q0), __ldg(c0 + 0));
  T.n1 = make_float4(__fmul_rn(v1.nx, q1), __fmul_rn(v1.ny, q1), __fmul_rn(v1.nz, q1), __ldg(c0 + 1));
  T.n2 = make_float4(__fmul_rn(v2.nx, q2), __fmul_rn(v2.ny, q2), __fmul_rn(v2.nz, q2), __ldg(c0 + 2));
  reinterpret_cast<TriSetup*>(p.setup)[slot] = T;
  if (p.persp) {
    TriPersp Q;
    Q.q = make_float4(q0, q1, q2, 0.0f);
    Q.vzq = make_float4(__fmul_rn(cv[0].vz, q0), __fmul_rn(v1.vz, q1), __fmul_rn(v2.vz, q2), 0.0f);
    reinterpret_cast<TriPersp*>(p.persp)[slot] = Q;
  }
  p.bbox[slot] =
      make_uint2((uint32_t)bx0 | ((uint32_t)by0 << 16), ((uint32_t)bx1 | ((uint32_t)by1 << 16)) | second_bit);
  const int tx0 = bx0 / kTile, tx1 = bx1 / kTile, ty0 = by0 / kTile, ty1 = by1 / kTile;
  return (uint32_t)((tx1 - tx0 + 1) * (ty1 - ty0 + 1));
}

// Triangle t's clip-space vertices (object.vert.glsl:32-39) and colour.
// Flattened mesh: 10 floats per vertex, colour of the first vertex.
// Instanced: template vertex (6 floats) scaled by the instance's radius and
// moved to its centre, one multiply and one add each rounded (as a flattened
// copy of the template is built on the host), colour of the instance.
__device__ __forceinline__ const float* clip_vertices(const SetupParams& p, uint32_t t, ClipVert (&cv)[3]) {
  const uint32_t tg = p.first_triangle + t;
  const float* __restrict__ vtx = p.vertices;
  const float* inst = nullptr;
  uint32_t tri = tg;
  if (p.instances) {
    const uint32_t o = tg / p.template_triangles;
    tri = tg - o * p.template_triangles;
    inst = p.instances + 8 * (size_t)o;
  }
  const uint32_t i0 = __ldg(&p.indices[3 * (size_t)tri + 0]);
  const uint32_t i1 = __ldg(&p.indices[3 * (size_t)tri + 1]);
  const uint32_t i2 = __ldg(&p.indices[3 * (size_t)tri + 2]);
  const uint32_t vid[3] = {i0, i1, i2};
  // scene constants from device memory (every thread reads the same 80 bytes)
  float m[16], v[16];
  {
    const float4* sc = reinterpret_cast<const float4*>(p.scene);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 c = __ldg(sc + k);
      m[4 * k + 0] = c.x;
      m[4 * k + 1] = c.y;
      m[4 * k + 2] = c.z;
      m[4 * k + 3] = c.w;
    }
    // of the view matrix only row 2 (view-space z) is used: columns' z entries
#pragma unroll
    for (int k = 0; k < 4; ++k) v[4 * k + 2] = __ldg(p.scene + 16 + 4 * k + 2);
  }
  float4 ic = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
  if (inst) ic = __ldg(reinterpret_cast<const float4*>(inst));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* pv = inst ? vtx + 6 * (size_t)vid[k] : vtx + 10 * (size_t)vid[k];
    float x = __ldg(pv + 0), y = __ldg(pv + 1), z = __ldg(pv + 2);
    if (inst) {
      x = __fadd_rn(__fmul_rn(x, ic.w), ic.x);
      y = __fadd_rn(__fmul_rn(y, ic.w), ic.y);
      z = __fadd_rn(__fmul_rn(z, ic.w), ic.z);
    }
    cv[k].x = __fmaf_rn(m[0], x, __fmaf_rn(m[4], y, __fmaf_rn(m[8], z, m[12])));
    cv[k].y = __fmaf_rn(m[1], x, __fmaf_rn(m[5], y, __fmaf_rn(m[9], z, m[13])));
    cv[k].z = __fmaf_rn(m[2], x, __fmaf_rn(m[6], y, __fmaf_rn(m[10], z, m[14])));
    cv[k].w = __fmaf_rn(m[3], x, __fmaf_rn(m[7], y, __fmaf_rn(m[11], z, m[15])));
    cv[k].vz = __fmaf_rn(v[2], x, __fmaf_rn(v[6], y, __fmaf_rn(v[10], z, v[14])));
    cv[k].nx = __ldg(pv + 3);
    cv[k].ny = __ldg(pv + 4);
    cv[k].nz = __ldg(pv + 5);
  }
  return inst ? inst + 4 : vtx + 10 * (size_t)i0 + 6;  // color.rgba
}

// pair_count of a triangle the near plane crosses, between k_setup and
// k_setup_clip (no triangle overlaps 2^32 - 1 tiles)
constexpr uint32_t kClipPending = 0xFFFFFFFFu;

// One thread per triangle. Triangles wholly in front of the near plane, or
// wholly behind it (dropped by the clip-volume test), are set up here; a
// crossing triangle is marked for k_setup_clip, which keeps this kernel's
// vertices in registers and free of the clip's extra state.
__global__ void __launch_bounds__(256, 4) k_setup(SetupParams p, int S) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.num_triangles) return;
  ClipVert cv[3];
  const float* c0 = clip_vertices(p, t, cv);
  const int nin = (cv[0].z >= 0.0f) + (cv[1].z >= 0.0f) + (cv[2].z >= 0.0f);
  if (nin == 1 || nin == 2) {
    p.pair_count[t] = kClipPending;
    return;
  }
  p.pair_count[t] = setup_half(p, S, t, t >= p.opaque_from, cv, c0, false);
}

// A triangle k_setup marked: Sutherland-Hodgman against z = 0 over the edges
// 0->1, 1->2, 2->0 keeps the triangle's winding; 3 vertices give one triangle
// (record t), 4 the fan (0, 1, 2) in record t and (0, 2, 3) in record
// num_triangles + t. The vertices are derived from the mesh again, with the
// same rounded operations as in k_setup. Returns the pair count.
__device__ __forceinline__ uint32_t setup_clipped(const SetupParams& p, int S, uint32_t t) {
  ClipVert cv[3];
  const float* c0 = clip_vertices(p, t, cv);
  const bool opaque = t >= p.opaque_from;
  const bool in[3] = {cv[0].z >= 0.0f, cv[1].z >= 0.0f, cv[2].z >= 0.0f};
  // the polygon: in-front vertices and edge cuts in edge order (3 or 4 of them)
  ClipVert poly[4];
  int n = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int k1 = k == 2 ? 0 : k + 1;
    if (in[k] && n < 4) poly[n++] = cv[k];
    if (in[k] != in[k1] && n < 4) poly[n++] = near_cut(cv[k], cv[k1]);
  }
  uint32_t pairs = 0;
  if (n >= 3) {
    const ClipVert first[3] = {poly[0], poly[1], poly[2]};
    pairs = setup_half(p, S, t, opaque, first, c0, n == 4);
    if (n == 4) {
      const ClipVert second[3] = {poly[0], poly[2], poly[3]};
      pairs += setup_half(p, S, p.num_triangles + t, opaque, second, c0, false);
    }
  } else {
    p.bbox[t] = make_uint2(0xFFFFFFFFu, 0u);  // not reached: a crossing triangle gives 3 or 4
  }
  p.pair_count[t] = pairs;
  return pairs;
}

// Triangles per block of the clip kernel (4 per thread) and of the emit
// kernel (one per thread): the pair-count sums are per 512 triangles.
constexpr int kClipThreads = 128;
constexpr int kEmitItems = 4;
constexpr int kEmitTile = kClipThreads * kEmitItems;

// The marked triangles of each 512-triangle block are clipped one by one;
// with block_sums, the block's pair count (after clipping) is written there,
// the first level of the pair-offset scan. pair_count is 16-byte aligned.
__global__ void __launch_bounds__(kClipThreads) k_setup_clip(SetupParams p, int S, uint32_t* __restrict__ block_sums) {
  __shared__ uint32_t warp_sums[kClipThreads / 32];
  const uint32_t n = p.num_triangles;
  const uint32_t t0 = blockIdx.x * kEmitTile + threadIdx.x * kEmitItems;
  uint32_t c[kEmitItems] = {0u, 0u, 0u, 0u};
  if (t0 + 3 < n) {
    const uint4 v = __ldcg(reinterpret_cast<const uint4*>(p.pair_count + t0));
    c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
  } else {
#pragma unroll
    for (int k = 0; k < kEmitItems; ++k) c[k] = t0 + k < n ? p.pair_count[t0 + k] : 0u;
  }
  uint32_t sum = 0;
#pragma unroll 1
  for (int k = 0; k < kEmitItems; ++k) {
    const uint32_t ck = c[k] == kClipPending ? setup_clipped(p, S, t0 + (uint32_t)k) : c[k];
    sum += ck;
  }
  if (!block_sums) return;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t b = 0;
#pragma unroll
    for (int w = 0; w < kClipThreads / 32; ++w) b += warp_sums[w];
    block_sums[blockIdx.x] = b;
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan (u32), 4096 elements per block, recursive over block sums.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total, uint32_t* smem) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t w = lane < nw ? smem[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    smem[32 + lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const uint32_t warp_prefix = warp ? smem[32 + warp - 1] : 0u;
  *total = smem[32 + (blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(const uint32_t* __restrict__ in, size_t n,
                                                            uint32_t* __restrict__ sums) {
  __shared__ uint32_t smem[64];
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += in[base + i];
  uint32_t total;
  block_exclusive_scan(s, &total, smem);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                             size_t n, const uint32_t* __restrict__ offsets,
                                                             uint32_t* __restrict__ grand_total) {
  __shared__ uint32_t smem[64];
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t total;
  uint32_t pre = block_exclusive_scan(s, &total, smem) + (offsets ? offsets[blockIdx.x] : 0u);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
  if (grand_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1) *grand_total = pre;
}

// One block walks the tiles of a short array in order, carrying the running
// sum: one launch instead of three for up to kScanLoopTiles tiles.
constexpr int kScanLoopTiles = 8;

__global__ void __launch_bounds__(kScanThreads) k_scan_loop(const uint32_t* __restrict__ in,
                                                            uint32_t* __restrict__ out, size_t n,
                                                            uint32_t* __restrict__ grand_total) {
  __shared__ uint32_t smem[64];
  uint32_t carry = 0;
  for (size_t tile = 0; tile * kScanTile < n; ++tile) {
    const size_t base = tile * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
      v[i] = (base + i < n) ? in[base + i] : 0u;
      s += v[i];
    }
    uint32_t total;
    uint32_t pre = block_exclusive_scan(s, &total, smem) + carry;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
      if (base + i < n) out[base + i] = pre;
      pre += v[i];
    }
    carry += total;
  }
  if (grand_total && threadIdx.x == 0) *grand_total = carry;
}

size_t blocks_for(size_t n) { return (n + kScanTile - 1) / kScanTile; }

// Exclusive scan of n u32 values; grand_total (device, may be null) receives the sum.
cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp, uint32_t* grand_total,
                           cudaStream_t s, uint64_t* launches) {
  if (n == 0) {
    if (grand_total) return cudaMemsetAsync(grand_total, 0, 4, s);
    return cudaSuccess;
  }
  const size_t nb = blocks_for(n);
  if (nb == 1) {
    k_scan_apply<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, grand_total);
    ++*launches;
    return cudaGetLastError();
  }
  if (nb <= (size_t)kScanLoopTiles) {
    k_scan_loop<<<1, kScanThreads, 0, s>>>(in, out, n, grand_total);
    ++*launches;
    return cudaGetLastError();
  }
  uint32_t* sums = tmp;
  uint32_t* rest = tmp + nb;
  k_scan_sums<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, sums);
  ++*launches;
  cudaError_t e = scan_exclusive(sums, sums, nb, rest, nullptr, s, launches);
  if (e != cudaSuccess) return e;
  k_scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, sums, grand_total);
  ++*launches;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Pair emission: pair j of triangle t lands at pair_offset[t] + j.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t emit_bbox(uint2 bb, uint32_t t, uint32_t tile_base, int tiles_x, uint32_t off,
                                              uint32_t j, uint32_t* __restrict__ keys, uint32_t* __restrict__ tris,
                                              size_t capacity) {
  const int bx0 = bb.x & 0xFFFF, by0 = bb.x >> 16, bx1 = bb.y & 0xFFFF, by1 = (bb.y >> 16) & 0x7FFF;
  if (bx0 > bx1 || by0 > by1) return j;
  const int tx0 = bx0 / kTile, ty0 = by0 / kTile, tx1 = bx1 / kTile, ty1 = by1 / kTile;
  for (int ty = ty0; ty <= ty1; ++ty) {
    // rows of 8x4 micro-tiles the bbox overlaps in this tile row
    const int ly0 = max(by0 - ty * kTile, 0), ly1 = min(by1 - ty * kTile, kTile - 1);
    uint32_t rows = 0;
    for (int r = ly0 >> 2; r <= (ly1 >> 2); ++r) rows |= 3u << (2 * r);
    for (int tx = tx0; tx <= tx1; ++tx, ++j) {
      const size_t pos = (size_t)off + j;
      if (pos >= capacity) return j;
      const int lx0 = max(bx0 - tx * kTile, 0), lx1 = min(bx1 - tx * kTile, kTile - 1);
      const uint32_t cols = (lx0 <= 7 ? 0x55u : 0u) | (lx1 >= 8 ? 0xAAu : 0u);
      keys[pos] = (tile_base + (uint32_t)(ty * tiles_x + tx)) | ((rows & cols) << kMaskShift);
      tris[pos] = t;
    }
  }
  return j;
}

// The pairs of the block's 512 triangles, one per thread: a triangle's
// offset is the scanned block sum plus the exclusive prefix of the counts
// before it in the block (written to pair_offset, which the bin-overflow walk
// reads); it emits its first (or only) half's tiles, then the second half's
// (record n + t) when the near-plane clip split it.
__global__ void __launch_bounds__(kEmitTile) k_emit(const uint32_t* __restrict__ pair_count,
                                                    uint32_t* __restrict__ pair_offset,
                                                    const uint32_t* __restrict__ block_offsets,
                                                    const uint2* __restrict__ bbox, uint32_t n, int tiles_x,
                                                    uint32_t opaque_from, uint32_t num_tiles,
                                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ tris,
                                                    size_t capacity, const uint32_t* __restrict__ total,
                                                    uint32_t* err) {
  __shared__ uint32_t smem[64];
  if (blockIdx.x == 0 && threadIdx.x == 0 && *total > capacity) atomicOr(err, 1u);  // OIT_DEVERR_BIN_OVERFLOW
  const uint32_t t = blockIdx.x * kEmitTile + threadIdx.x;
  const uint32_t c = t < n ? __ldg(&pair_count[t]) : 0u;
  uint32_t block_total;
  const uint32_t off = block_exclusive_scan(c, &block_total, smem) + block_offsets[blockIdx.x];
  if (t >= n) return;
  pair_offset[t] = off;
  if (!c) return;
  const uint2 bb = bbox[t];
  const uint32_t tile_base = t < opaque_from ? num_tiles : 0u;
  const uint32_t j = emit_bbox(bb, t, tile_base, tiles_x, off, 0u, keys, tris, capacity);
  if (bb.y >> 31) emit_bbox(bbox[n + t], n + t, tile_base, tiles_x, off, j, keys, tris, capacity);
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (key, value) pairs, 8-bit digits.
//
// The pairs are cut into at most kSortBlocks chunks (multiples of 2048
// pairs). k_radix_hist counts each chunk's digits; k_radix_scatter derives
// its chunk's output offset for every digit from those counts itself (the
// digit's start over all chunks plus the counts of the chunks before it) and
// moves the chunk 2048 pairs at a time: each warp ranks its 256 consecutive
// pairs with its own shared-memory counters, so a sub-tile costs three block
// barriers. Pairs keep their order within a digit: the sort is stable.
// ---------------------------------------------------------------------------
__device__ __forceinline__ size_t pair_count_of(const uint32_t* total, size_t capacity) {
  const size_t t = *total;
  return t < capacity ? t : capacity;
}

constexpr int kSortSubTile = kRadixThreads * kRadixRounds;  // 2048 pairs: 8 warps x 8 rounds of 32
constexpr int kSortWarps = kRadixThreads / 32;

// Digit counts of chunk blockIdx.x: counts[chunk * 256 + digit], or, with
// digit_major (many chunks, scanned in place before the scatter),
// counts[digit * gridDim.x + chunk]. One shared-memory atomic per distinct
// digit per warp (tile ids of neighbouring pairs are mostly equal).
__global__ void __launch_bounds__(kRadixThreads) k_radix_hist(const uint32_t* __restrict__ keys,
                                                              const uint32_t* __restrict__ total, size_t capacity,
                                                              int shift, size_t chunk, bool digit_major,
                                                              uint32_t* __restrict__ counts) {
  __shared__ uint32_t h[kRadixBins];
  h[threadIdx.x] = 0;
  __syncthreads();
  const size_t n = pair_count_of(total, capacity);
  const size_t beg = (size_t)blockIdx.x * chunk;
  const size_t end = beg + chunk < n ? beg + chunk : n;
  const uint32_t lane = threadIdx.x & 31;
  for (size_t base = beg; base < end; base += kRadixThreads * 4) {
    uint32_t d[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const size_t i = base + (size_t)k * kRadixThreads + threadIdx.x;
      d[k] = i < end ? (__ldg(&keys[i]) >> shift) & (kRadixBins - 1) : kRadixBins;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t peers = __match_any_sync(0xffffffffu, d[k]);
      if (d[k] < kRadixBins && (__ffs(peers) - 1) == (int)lane) atomicAdd(&h[d[k]], (uint32_t)__popc(peers));
    }
  }
  __syncthreads();
  if (digit_major) counts[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
  else counts[(size_t)blockIdx.x * kRadixBins + threadIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(const uint32_t* __restrict__ keys_in,
                                                                 const uint32_t* __restrict__ vals_in,
                                                                 uint32_t* __restrict__ keys_out,
                                                                 uint32_t* __restrict__ vals_out,
                                                                 const uint32_t* __restrict__ total, size_t capacity,
                                                                 int shift, size_t chunk, uint32_t nchunks,
                                                                 bool scanned, const uint32_t* __restrict__ counts) {
  __shared__ uint32_t base[kRadixBins];             // output position of the chunk's next pair of each digit
  __shared__ uint32_t wcount[kSortWarps][kRadixBins];  // per warp: counts, then exclusive offsets in the sub-tile
  __shared__ uint32_t sub_total[kRadixBins];
  __shared__ uint32_t scan_s[64];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const size_t n = pair_count_of(total, capacity);
  const size_t beg = (size_t)blockIdx.x * chunk;
  // this digit's pairs in all chunks, and in the chunks before this one
  if (scanned) {
    // the digit-major counts, scanned: this chunk's output offset per digit
    base[threadIdx.x] = __ldg(&counts[(size_t)threadIdx.x * nchunks + blockIdx.x]);
    __syncthreads();
  } else {
    // 32 independent loads in flight per thread: the chunks' counts are read
    // by every block, so their latency, not their bytes, is the cost
    const uint32_t d = threadIdx.x;
    uint32_t all = 0, before = 0;
    for (uint32_t c0 = 0; c0 < nchunks; c0 += 32) {
      uint32_t v[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] = c0 + k < nchunks ? __ldg(&counts[(size_t)(c0 + k) * kRadixBins + d]) : 0u;
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        all += v[k];
        before += c0 + k < blockIdx.x ? v[k] : 0u;
      }
    }
    uint32_t sum_all;
    base[d] = block_exclusive_scan(all, &sum_all, scan_s) + before;
  }
  if (beg >= n) return;
  const size_t end = beg + chunk < n ? beg + chunk : n;
  for (size_t sub = beg; sub < end; sub += kSortSubTile) {
#pragma unroll
    for (int k = 0; k < kRadixBins / 32; ++k) wcount[warp][lane + 32 * k] = 0;
    __syncwarp();
    // this warp's 256 consecutive pairs of the sub-tile, 32 per round
    const size_t wbase = sub + (size_t)warp * (32 * kRadixRounds);
    uint32_t key[kRadixRounds], val[kRadixRounds], dr[kRadixRounds];
#pragma unroll
    for (int r = 0; r < kRadixRounds; ++r) {
      const size_t i = wbase + (size_t)r * 32 + lane;
      key[r] = i < end ? __ldg(&keys_in[i]) : 0u;
      val[r] = i < end ? __ldg(&vals_in[i]) : 0u;
    }
#pragma unroll
    for (int r = 0; r < kRadixRounds; ++r) {
      const size_t i = wbase + (size_t)r * 32 + lane;
      const uint32_t d = i < end ? (key[r] >> shift) & (kRadixBins - 1) : kRadixBins;
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const int leader = __ffs(peers) - 1;
      uint32_t old = 0;
      if (lane == leader && d < kRadixBins) {
        old = wcount[warp][d];
        wcount[warp][d] = old + (uint32_t)__popc(peers);
      }
      old = __shfl_sync(0xffffffffu, old, leader);
      dr[r] = (d << 16) | (old + (uint32_t)__popc(peers & lt_mask));  // digit (256 = none), rank in the warp
    }
    __syncthreads();
    {
      const int d = threadIdx.x;
      uint32_t acc = 0;
#pragma unroll
      for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = wcount[w][d];
        wcount[w][d] = acc;
        acc += c;
      }
      sub_total[d] = acc;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRadixRounds; ++r) {
      const uint32_t d = dr[r] >> 16;
      if (d < kRadixBins) {
        const uint32_t pos = base[d] + wcount[warp][d] + (dr[r] & 0xFFFFu);
        keys_out[pos] = key[r];
        vals_out[pos] = val[r];
      }
    }
    __syncthreads();
    base[threadIdx.x] += sub_total[threadIdx.x];
  }
}

// [begin, end) of every tile's pair range in the sorted keys: every position
// where the key changes ends the previous key's range and begins the next
// one's. Both arrays start at zero, so tiles without pairs read an empty range.
__global__ void __launch_bounds__(256) k_tile_bounds(const uint32_t* __restrict__ keys,
                                                     const uint32_t* __restrict__ total, size_t capacity,
                                                     uint32_t num_keys, uint32_t* __restrict__ begin,
                                                     uint32_t* __restrict__ end) {
  const uint32_t n = (uint32_t)pair_count_of(total, capacity);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    const uint32_t cur = i < n ? keys[i] & kTileKeyMask : num_keys;
    const uint32_t prev = i > 0 ? keys[i - 1] & kTileKeyMask : 0xFFFFFFFFu;
    if (cur == prev) continue;
    if (i > 0 && prev < num_keys) end[prev] = i;
    if (cur < num_keys) begin[cur] = i;
  }
}

__global__ void k_fill_u32(uint32_t* dst, uint32_t v, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] = v;
}

__global__ void k_fill_f4(float4* dst, float4 v, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] = v;
}

}  // namespace

size_t scan_scratch_words(size_t n) {
  size_t words = 0;
  while (n > 1) {
    n = blocks_for(n);
    words += n;
  }
  return words + 1;
}

cudaError_t launch_fill_u32(uint32_t* dst, uint32_t value, size_t count, cudaStream_t s) {
  if (!count) return cudaSuccess;
  const unsigned blocks = (unsigned)std::min<size_t>((count + 255) / 256, 152 * 16);
  k_fill_u32<<<blocks, 256, 0, s>>>(dst, value, count);
  return cudaGetLastError();
}

cudaError_t launch_fill_f4(float4* dst, float4 value, size_t count, cudaStream_t s) {
  if (!count) return cudaSuccess;
  const unsigned blocks = (unsigned)std::min<size_t>((count + 255) / 256, 152 * 16);
  k_fill_f4<<<blocks, 256, 0, s>>>(dst, value, count);
  return cudaGetLastError();
}

namespace {
// k_setup, then k_setup_clip over the triangles it marked (and, with
// block_sums, the pair count of every 512-triangle block)
cudaError_t launch_setup(const SetupParams& sp, uint32_t* block_sums, cudaStream_t s, uint64_t* launches) {
  const uint32_t n = sp.num_triangles;
  const int S = sp.samples > 1 ? sp.samples : 1;
  k_setup<<<(n + 255) / 256, 256, 0, s>>>(sp, S);
  ++*launches;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_setup_clip<<<(unsigned)emit_blocks(n), kClipThreads, 0, s>>>(sp, S, block_sums);
  ++*launches;
  return cudaGetLastError();
}

// Pairs per chunk of the radix sort. Up to direct_max pairs: whole 2048-pair
// sub-tiles, at most kSortBlocks chunks, each scatter block summing the counts
// of the chunks before it. Beyond: one sub-tile per chunk (every block busy),
// the digit-major counts scanned in place.
constexpr size_t kSortBlocks = 128;
bool sort_scanned(size_t capacity, size_t direct_max) { return capacity > direct_max; }
size_t sort_chunk(size_t capacity, size_t direct_max) {
  if (sort_scanned(capacity, direct_max)) return kSortSubTile;
  const size_t per = (capacity + kSortBlocks - 1) / kSortBlocks;
  const size_t sub = (per + kSortSubTile - 1) / kSortSubTile * kSortSubTile;
  return sub > (size_t)kSortSubTile ? sub : (size_t)kSortSubTile;
}
}  // namespace

size_t emit_blocks(size_t tris) { return (tris + kEmitTile - 1) / kEmitTile; }

size_t bin_scan_words(size_t tris) {
  const size_t nb = emit_blocks(tris > 0 ? tris : 1);
  return nb + scan_scratch_words(nb);
}

cudaError_t bin_setup_only(const SetupParams& sp, cudaStream_t s, uint64_t* launches) {
  const uint32_t n = sp.num_triangles;
  if (n == 0) return cudaSuccess;
  return launch_setup(sp, nullptr, s, launches);
}

// Binning, step 1: setup, clip, pair counts per 512-triangle block and their
// exclusive scan (in b.scan_tmp, read by k_emit); the number of (tile,
// triangle) pairs lands in b.total (device).
cudaError_t bin_setup_scan(const SetupParams& sp, Bins& b, cudaStream_t s, uint64_t* launches) {
  cudaError_t e;
  const uint32_t n = sp.num_triangles;
  if (n == 0) return cudaMemsetAsync(b.total, 0, 4, s);
  if ((e = launch_setup(sp, b.scan_tmp, s, launches)) != cudaSuccess) return e;
  const size_t nb = emit_blocks(n);
  return scan_exclusive(b.scan_tmp, b.scan_tmp, nb, b.scan_tmp + nb, b.total, s, launches);
}

// Binning, step 2: emit pairs in triangle order, stable radix sort by tile id,
// tile ranges. Every kernel reads the pair count from b.total and is bounded
// by b.capacity, so no host round trip is needed; pairs beyond the capacity
// are dropped and raise OIT_DEVERR_BIN_OVERFLOW.
cudaError_t bin_sort(const SetupParams& sp, Bins& b, int key_bits, int num_tiles, uint32_t* error, cudaStream_t s,
                     uint64_t* launches) {
  cudaError_t e;
  const uint32_t n = sp.num_triangles;
  if (n > 0) {
    k_emit<<<(unsigned)emit_blocks(n), kEmitTile, 0, s>>>(sp.pair_count, b.pair_offset, b.scan_tmp, sp.bbox, n,
                                                          sp.tiles_x, sp.opaque_from, (uint32_t)sp.num_tiles, b.keys,
                                                          b.tris, b.capacity, b.total, error);
    ++*launches;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  const size_t chunk = sort_chunk(b.capacity, b.sort_direct_max);
  const uint32_t nchunks = (uint32_t)std::max<size_t>((b.capacity + chunk - 1) / chunk, 1);
  uint32_t *kin = b.keys, *vin = b.tris, *kout = b.keys_alt, *vout = b.tris_alt;
  const bool scanned = sort_scanned(b.capacity, b.sort_direct_max);
  for (int shift = 0; shift < key_bits; shift += kRadixBits) {
    k_radix_hist<<<nchunks, kRadixThreads, 0, s>>>(kin, b.total, b.capacity, shift, chunk, scanned, b.hist);
    ++*launches;
    if (scanned && (e = scan_exclusive(b.hist, b.hist, (size_t)nchunks * kRadixBins, b.hist + (size_t)nchunks * kRadixBins,
                                       nullptr, s, launches)) != cudaSuccess)
      return e;
    k_radix_scatter<<<nchunks, kRadixThreads, 0, s>>>(kin, vin, kout, vout, b.total, b.capacity, shift, chunk,
                                                      nchunks, scanned, b.hist);
    ++*launches;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  if (kin != b.keys) {
    std::swap(b.keys, b.keys_alt);
    std::swap(b.tris, b.tris_alt);
  }
  // ranges of both kinds: [0, num_tiles) opaque, [num_tiles, 2 num_tiles) transparent
  const size_t range_bytes = (size_t)2 * num_tiles * sizeof(uint32_t);
  if ((e = cudaMemsetAsync(b.tile_begin, 0, range_bytes, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(b.tile_end, 0, range_bytes, s)) != cudaSuccess) return e;
  const size_t nb = std::min<size_t>((b.capacity + 256) / 256, 152 * 16);
  k_tile_bounds<<<(unsigned)std::max<size_t>(nb, 1), 256, 0, s>>>(b.keys, b.total, b.capacity,
                                                                  (uint32_t)(2 * num_tiles), b.tile_begin,
                                                                  b.tile_end);
  ++*launches;
  return cudaGetLastError();
}

// Digit counts of the chunks (and, for the scanned sort, its scan scratch).
size_t radix_hist_words(size_t pairs, bool with_scanned) {
  const size_t direct = kSortBlocks * kRadixBins;
  if (!with_scanned) return direct;
  const size_t words = (pairs + kSortSubTile - 1) / kSortSubTile * kRadixBins;
  return std::max(direct, words + scan_scratch_words(words));
}

void srgb_host_tables(float* thr256, float* dec256) {
  static const float thr[256] = OIT_SRGB_THR_INIT;
  static const float dec[256] = OIT_SRGB_DEC_INIT;
  for (int i = 0; i < 256; ++i) {
    thr256[i] = thr[i];
    dec256[i] = dec[i];
  }
}

}  // namespace oit
