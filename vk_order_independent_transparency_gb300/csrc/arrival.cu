// Arrival-order linked-list COLOR pass (OIT_FLAG_ARRIVAL_ORDER).
//
// The reference's linked-list fragment shader (oitLinkedList.frag.glsl:51-85)
// as its GPU runs it: the fragments of all triangles in parallel, in whatever
// order they arrive. Each fragment takes a node from the global counter
// (imageAtomicAdd, :55; here one atomicAdd per warp round for the round's
// fragments) and links itself in front of its pixel's list by an atomic
// exchange of the head in HBM (imageAtomicExchange, :60-67). A fragment that
// finds the pool full is blended into the colour target (:71-83) under a
// per-pixel spinlock, in arrival order (lanes of one warp with the same pixel
// in lane order); the spin is bounded and a spin that gives up raises
// OIT_DEVERR_TIMEOUT instead of blending.
//
// Work: a warp takes 32 consecutive triangles of the pass and numbers the
// pixels of their bboxes (a prefix sum over the bbox areas); lane g of each
// round of 32 tests pixel g, so tiny triangles keep every lane busy. No tile
// binning is needed: the setup records and bboxes are the whole input.
#include <algorithm>

#include "../../include/oit_gb300.h"
#include "oit_device.cuh"
#include "oit_internal.h"

namespace oit {
using namespace oitd;

namespace {

constexpr int kArrivalWarps = 8;
constexpr uint32_t kFullMask = 0xffffffffu;
constexpr int kSpinLimit = 1 << 20;

// dst = src over dst on the colour target element, under the pixel's lock.
__device__ __forceinline__ bool locked_tail_blend(const ArrivalParams& p, uint32_t pixel, const float4& src) {
  for (int it = 0; it < kSpinLimit; ++it) {
    if (atomicCAS(&p.locks[pixel], 0u, 1u) == 0u) {
      __threadfence();
      float4 c;
      if (p.color_half) {
        const uint2 v = __ldcg(reinterpret_cast<const uint2*>(p.color) + pixel);
        const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
        const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
        c = make_float4(lo.x, lo.y, hi.x, hi.y);
      } else {
        c = __ldcg(p.color + pixel);
      }
      rop_over(c, src);
      if (p.color_half) {
        const __half2 lo = __floats2half2_rn(c.x, c.y), hi = __floats2half2_rn(c.z, c.w);
        __stcg(reinterpret_cast<uint2*>(p.color) + pixel,
               make_uint2(*reinterpret_cast<const uint32_t*>(&lo), *reinterpret_cast<const uint32_t*>(&hi)));
      } else {
        __stcg(p.color + pixel, c);
      }
      __threadfence();
      atomicExch(&p.locks[pixel], 0u);
      return true;
    }
  }
  return false;
}

__global__ void __launch_bounds__(32 * kArrivalWarps, 4) k_arrival_ll(ArrivalParams p) {
  __shared__ unsigned long long pre_s[kArrivalWarps][32];  // exclusive prefix of the bbox areas
  __shared__ uint4 geo_s[kArrivalWarps][32];               // bbox x0, y0, width; triangle
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  unsigned long long* pre = pre_s[warp];
  uint4* geo = geo_s[warp];
  const TriSetup* __restrict__ setup = reinterpret_cast<const TriSetup*>(p.setup);
  const uint32_t stride = gridDim.x * kArrivalWarps * 32u;
  uint32_t nfrag = 0;  // warp-uniform
  // entries [0, n): records 0 .. n-1; entries [n, 2n): the second halves of
  // near-clipped triangles, records second_base + 0 .. n-1
  for (uint32_t base = (blockIdx.x * kArrivalWarps + warp) * 32u; base < 2u * p.num_tris; base += stride) {
    const uint32_t v = base + lane;
    const bool second = v >= p.num_tris;
    const uint32_t t = second ? p.second_base + (v - p.num_tris) : v;
    uint32_t x0 = 0, y0 = 0, wd = 1;
    unsigned long long area = 0;
    if (v < 2u * p.num_tris && (!second || (__ldg(&p.bbox[v - p.num_tris]).y >> 31))) {
      const uint2 bb = __ldg(&p.bbox[t]);
      const int bx0 = bb.x & 0xFFFF, by0 = bb.x >> 16, bx1 = bb.y & 0xFFFF, by1 = (bb.y >> 16) & 0x7FFF;
      if (bx0 <= bx1 && by0 <= by1) {  // culled triangles carry an empty bbox
        x0 = (uint32_t)bx0;
        y0 = (uint32_t)by0;
        wd = (uint32_t)(bx1 - bx0 + 1);
        area = (unsigned long long)wd * (unsigned long long)(by1 - by0 + 1);
      }
    }
    unsigned long long incl = area;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(kFullMask, incl, o);
      if (lane >= o) incl += y;
    }
    const unsigned long long total = __shfl_sync(kFullMask, incl, 31);
    pre[lane] = incl - area;
    geo[lane] = make_uint4(x0, y0, wd, t);
    __syncwarp();
    for (unsigned long long g0 = 0; g0 < total; g0 += 32) {
      const unsigned long long g = g0 + lane;
      bool frag = false;
      uint32_t pixel = 0, zbits = 0, tri = 0;
      int px = 0, py = 0;
      if (g < total) {
        // the triangle holding pixel g: the last one whose prefix is <= g
        int lo = 0, hi = 31;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (pre[mid] <= g) lo = mid; else hi = mid - 1;
        }
        const uint4 gm = geo[lo];
        const uint32_t r = (uint32_t)(g - pre[lo]);
        const uint32_t row = r / gm.z;
        px = (int)(gm.x + (r - row * gm.z));
        py = (int)(gm.y + row);
        tri = gm.w;
        const TriSetup& T = setup[tri];
        const int4 a = T.xy01, b = T.xy2f;
        const float4 zc = T.zc;
        const int sx = px * 256 + 128, sy = py * 256 + 128;
        float z = 0.f;
        bool in;
        if (b.z & kFlagSmall) {
          const EdgesT<int> e = edges_at<int>(a, b, sx, sy);
          in = inside(e, b.z);
          if (in) z = depth_at(zc, e);
        } else {
          const EdgesT<long long> e = edges_at<long long>(a, b, sx, sy);
          in = inside(e, b.z);
          if (in) z = depth_at(zc, e);
        }
        if (in) {
          pixel = (uint32_t)py * (uint32_t)p.RW + (uint32_t)px;
          const uint32_t od = p.has_opaque ? __ldg(&p.depth[pixel]) : 0x3F800000u;  // early depth test
          zbits = __float_as_uint(z);
          frag = zbits < od;
        }
      }
      const uint32_t m = __ballot_sync(kFullMask, frag);
      if (!m) continue;
      uint32_t node0 = 0;
      if (lane == __ffs(m) - 1) node0 = atomicAdd(p.counter, (uint32_t)__popc(m));
      node0 = __shfl_sync(kFullMask, node0, __ffs(m) - 1);
      bool pending = false;  // a tail blend to make
      float4 src = make_float4(0.f, 0.f, 0.f, 0.f);
      if (frag) {
        const TriSetup& T = setup[tri];
        const int4 a = T.xy01, b = T.xy2f;
        const int sx = px * 256 + 128, sy = py * 256 + 128;
        Shade sh;
        if (b.z & kFlagSmall) sh = shade(T, edges_at<int>(a, b, sx, sy), nullptr);
        else sh = shade(T, edges_at<long long>(a, b, sx, sy), nullptr);
        const uint32_t node = node0 + 1u + (uint32_t)__popc(m & lt);
        if (node < p.capacity) {
          const uint32_t packed = pack_rgba8(sh, (uint32_t)(b.z >> 8) & 255u);
          const uint32_t old = atomicExch(&p.heads[pixel], node);
          reinterpret_cast<uint4*>(p.pool)[node] = make_uint4(packed, zbits, 0u, old);
        } else if (p.tail) {
          const float al = __int_as_float(b.w);
          src = make_float4(sh.r * al, sh.g * al, sh.b * al, al);
          pending = true;
        }
      }
      // Tail blends: lanes of one warp that share a pixel take its lock one at
      // a time, lowest lane (earliest node) first, so a lock is only ever
      // contended by other warps, which run independently.
      while (__any_sync(kFullMask, pending)) {
        const uint32_t peers = __match_any_sync(kFullMask, pending ? pixel : 0xFFFFFFFFu);
        if (pending && lane == __ffs(peers) - 1) {
          if (!locked_tail_blend(p, pixel, src)) atomicOr(p.error, OIT_DEVERR_TIMEOUT);
          pending = false;
        }
      }
      nfrag += (uint32_t)__popc(m);
    }
    __syncwarp();  // the next chunk overwrites pre / geo
  }
  if (lane == 0 && nfrag) atomicAdd(p.frag_count, (unsigned long long)nfrag);
}

// The colour target before the pass: the opaque colour (or the background).
__global__ void k_arrival_init(ArrivalParams p) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < p.P; i += gridDim.x * blockDim.x) {
    const float4 c = p.has_opaque ? p.opaque_color[i] : p.background;
    store_color(p.color, p.color_half != 0, i, c);
    p.heads[i] = 0u;
    p.locks[i] = (int32_t)i == p.held_lock ? 1u : 0u;  // a held lock is never released
  }
}

}  // namespace

cudaError_t launch_arrival_ll(const ArrivalParams& p, cudaStream_t s, uint64_t* launches) {
  if (p.P) {
    const unsigned blocks = (unsigned)std::min<size_t>(((size_t)p.P + 255) / 256, 152 * 16);
    k_arrival_init<<<blocks, 256, 0, s>>>(p);
    ++*launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (p.num_tris) {
    const size_t warps = (2 * (size_t)p.num_tris + 31) / 32;
    const unsigned blocks = (unsigned)std::min<size_t>((warps + kArrivalWarps - 1) / kArrivalWarps, 152 * 16);
    k_arrival_ll<<<blocks, 32 * kArrivalWarps, 0, s>>>(p);
    ++*launches;
  }
  return cudaGetLastError();
}

}  // namespace oit
