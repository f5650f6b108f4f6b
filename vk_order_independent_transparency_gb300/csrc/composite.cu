// COMPOSITE pass fused with the back-buffer copy.
//
// One thread per output pixel: gathers the pixel's A-buffer entries, sorts
// them exactly as the reference's composite shader does (bubbleSort with its
// swap-on-equal, insertionSortTail for linked-list tails), blends front to
// back in FP32, applies the blend onto the tail-blended colour target
// (ONE, ONE_MINUS_SRC_ALPHA, main.cpp:548-558), then resolves MSAA samples /
// supersampled pixels with a box filter and encodes sRGB8 once
// (copyOffscreenToBackBuffer, main.cpp:645-774). Sort arrays are register
// arrays with compile-time OIT_LAYERS, so every index is static.
#include <cuda_fp16.h>

#include "list_walk.cuh"
#include "oit_device.cuh"
#include "oit_internal.h"

namespace oit {
using namespace oitd;

namespace {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;

__device__ __forceinline__ bool dge(uint32_t a, uint32_t b) { return __uint_as_float(a) >= __uint_as_float(b); }
__device__ __forceinline__ bool dlt(uint32_t a, uint32_t b) { return __uint_as_float(a) < __uint_as_float(b); }

template <int L>
struct Arr {
  uint32_t c[L], d[L], m[L];
};

// bubbleSort, shaders/oitCompositeDefines.glsl:51-89: swaps on >=.
template <int L>
__device__ __forceinline__ void bubble_sort(Arr<L>& a, int n) {
#pragma unroll
  for (int i = L - 2; i >= 0; --i) {
    if (i <= n - 2) {
#pragma unroll
      for (int j = 0; j <= i; ++j) {
        if (dge(a.d[j], a.d[j + 1])) {
          uint32_t t;
          t = a.c[j]; a.c[j] = a.c[j + 1]; a.c[j + 1] = t;
          t = a.d[j]; a.d[j] = a.d[j + 1]; a.d[j + 1] = t;
          t = a.m[j]; a.m[j] = a.m[j + 1]; a.m[j + 1] = t;
        }
      }
    }
  }
}

// insertionSort / insertionSortTail, oitCompositeDefines.glsl:94-139, on a
// full array of L entries. Returns the evicted entry's colour (the item itself
// when it is not nearer than the last entry).
template <int L>
__device__ __forceinline__ uint32_t insertion_sort_tail(Arr<L>& a, uint32_t ic, uint32_t id, uint32_t im) {
  if (!dlt(id, a.d[L - 1])) return ic;
  const uint32_t last = a.c[L - 1];
#pragma unroll
  for (int i = L - 1; i >= 1; --i) {
    if (dlt(id, a.d[i - 1])) {
      a.c[i] = a.c[i - 1]; a.d[i] = a.d[i - 1]; a.m[i] = a.m[i - 1];
    } else if (dlt(id, a.d[i])) {
      a.c[i] = ic; a.d[i] = id; a.m[i] = im;
    }
  }
  if (dlt(id, a.d[0])) {
    a.c[0] = ic; a.d[0] = id; a.m[0] = im;
  }
  return last;
}

// Premultiplied colour of an array entry: the packed RGBA8 record itself, or
// (RGBA32F linked-list nodes) the float colour of the node the entry names.
struct PackedColour {
  __device__ __forceinline__ float4 operator()(uint32_t c) const { return decode_premult(c); }
};
struct NodeColour {
  const uint4* pool;
  __device__ __forceinline__ float4 operator()(uint32_t node) const {
    const uint4 v = pool[2 * (size_t)node];
    const float a = __uint_as_float(v.w);
    return make_float4(__uint_as_float(v.x) * a, __uint_as_float(v.y) * a, __uint_as_float(v.z) * a, a);
  }
};

template <int L, class Col = PackedColour>
__device__ __forceinline__ float4 blend_array(const Arr<L>& a, int n, int coverage, int S, Col col = Col()) {
  float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!coverage) {
#pragma unroll
    for (int i = 0; i < L; ++i)
      if (i < n) blend_under(sum, col(a.c[i]));
    return sum;
  }
  // oitSimple.frag.glsl:142-159: per MSAA sample, blend the fragments covering it.
  for (int s = 0; s < S; ++s) {
    float4 sc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int i = 0; i < L; ++i)
      if (i < n && ((a.m[i] >> s) & 1u)) blend_under(sc, col(a.c[i]));
    sum.x += sc.x; sum.y += sc.y; sum.z += sc.z; sum.w += sc.w;
  }
  const float k = 1.0f / (float)S;
  return make_float4(sum.x * k, sum.y * k, sum.z * k, sum.w * k);
}

// Simple / Spinlock / Interlock: oitSimple.frag.glsl:115-169 (the Spinlock and
// Interlock composites, oitSpinlock.frag.glsl:153-207 and
// oitInterlock.frag.glsl:384-438, are identical).
template <int L>
__device__ __forceinline__ float4 composite_records(const CompositeParams& p, uint32_t eaux, size_t abase) {
  int n = (int)min(p.aux[eaux], (uint32_t)L);
  Arr<L> a;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    a.c[i] = 0; a.d[i] = 0; a.m[i] = 0;
    if (i < n) {
      const size_t o = abase + (size_t)i * p.P;
      if (p.coverage) {
        const uint4 r = reinterpret_cast<const uint4*>(p.abuf)[o];
        a.c[i] = r.x; a.d[i] = r.y; a.m[i] = r.z;
      } else {
        const uint2 r = reinterpret_cast<const uint2*>(p.abuf)[o];
        a.c[i] = r.x; a.d[i] = r.y;
      }
    }
  }
  bubble_sort<L>(a, n);
  return blend_array<L>(a, n, p.coverage, p.S);
}

// Linked list: oitLinkedList.frag.glsl:106-172. With RGBA32F records (F32)
// nodes are 32 bytes and the sort arrays carry node indices; colours are
// fetched when blended.
template <int L, bool F32>
__device__ __forceinline__ float4 composite_list(const CompositeParams& p, uint32_t eaux) {
  const uint4* __restrict__ pool = reinterpret_cast<const uint4*>(p.abuf);
  uint32_t off = p.aux[eaux];
  if (off >= p.capacity) off = 0;
  int n = 0;
  Arr<L> a;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    a.c[i] = 0; a.d[i] = 0; a.m[i] = 0;
    if (off != 0 && off < p.capacity) {
      if (F32) {
        const uint4 nd = pool[2 * (size_t)off + 1];  // depth, mask, next
        a.c[i] = off; a.d[i] = nd.x; a.m[i] = nd.y;
        off = nd.z;
      } else {
        const uint4 nd = pool[off];
        a.c[i] = nd.x; a.d[i] = nd.y; a.m[i] = nd.z;
        off = nd.w;
      }
      n = i + 1;
    }
  }
  bubble_sort<L>(a, n);
  float4 tail = make_float4(0.f, 0.f, 0.f, 0.f);
  // Lists built by the COLOR pass strictly decrease in node index; the bound
  // only guards against a list that was never built this frame.
  uint32_t guard = p.capacity;
  while (off != 0 && off < p.capacity && guard-- != 0) {
    uint32_t ic, id, im, next;
    if (F32) {
      const uint4 nd = pool[2 * (size_t)off + 1];
      ic = off; id = nd.x; im = nd.y; next = nd.z;
    } else {
      const uint4 nd = pool[off];
      ic = nd.x; id = nd.y; im = nd.z; next = nd.w;
    }
    const uint32_t ev = insertion_sort_tail<L>(a, ic, id, im);
    if (p.tail) blend_under(tail, F32 ? NodeColour{pool}(ev) : decode_premult(ev));
    off = next;
  }
  float4 sum = F32 ? blend_array<L>(a, n, p.coverage, p.S, NodeColour{pool}) : blend_array<L>(a, n, p.coverage, p.S);
  blend_under(sum, tail);
  return sum;
}

// Linked list per pixel: register sort arrays for OIT_LAYERS <= 8; beyond,
// the local-array walk (list_walk.cuh), whose register use does not grow with
// OIT_LAYERS (register arrays of 16 or 32 entries cost one or two resident
// blocks per SM on a latency-bound pointer chase).
template <int L, bool F32>
__device__ __forceinline__ float4 list_pixel(const CompositeParams& p, uint32_t eaux) {
  if (L <= 8) return composite_list<L, F32>(p, eaux);
  const uint4* __restrict__ pool = reinterpret_cast<const uint4*>(p.abuf);
  const uint32_t head = p.aux[eaux];
  if (p.coverage) {
    WalkArrays<true> a;
    return walk_list<F32>(pool, head, p.capacity, L, p.tail, p.S, a);
  }
  WalkArrays<false> a;
  return walk_list<F32>(pool, head, p.capacity, L, p.tail, p.S, a);
}

// Loop32: oitLoop.frag.glsl:191-222.
__device__ __forceinline__ float4 composite_loop(const CompositeParams& p, size_t abase) {
  int n = 0;
  for (int i = 0; i < p.L; ++i) {
    if (p.abuf[abase + (size_t)i * p.P] != kEmpty) n++; else break;
  }
  float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i = 0; i < n; ++i) blend_under(sum, decode_premult(p.abuf[abase + (size_t)(p.L + i) * p.P]));
  return sum;
}

// Loop64: oitLoop64.frag.glsl:162-183.
// With RGBA32F records a float4 payload block follows the keys.
__device__ __forceinline__ float4 composite_loop64(const CompositeParams& p, size_t abase) {
  const uint2* __restrict__ ab = reinterpret_cast<const uint2*>(p.abuf);
  const float4* __restrict__ pay =
      p.record_fp32 ? reinterpret_cast<const float4*>(ab + (size_t)p.ssn * p.L * p.P) : nullptr;
  float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i = 0; i < p.L; ++i) {
    const uint2 k = ab[abase + (size_t)i * p.P];
    if (k.y == kEmpty) break;
    if (pay) {
      const float4 c = pay[abase + (size_t)i * p.P];
      blend_under(sum, make_float4(c.x * c.w, c.y * c.w, c.z * c.w, c.w));
    } else {
      blend_under(sum, decode_premult(k.x));
    }
  }
  return sum;
}

__device__ __forceinline__ void write_out(const CompositeParams& p, uint32_t o, float4 c) {
  write_rgba8(p.out_rgba8, p.out_linear, o, c);
}

enum Kind { kRecords = 0, kList = 1, kLoop = 2, kLoop64 = 3, kListF32 = 4 };

template <int K, int L>
__global__ void __launch_bounds__(256) k_composite(CompositeParams p) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= p.W || y >= p.H) return;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int dy = 0; dy < p.ss; ++dy)
    for (int dx = 0; dx < p.ss; ++dx) {
      const uint32_t pixel = (uint32_t)(y * p.ss + dy) * (uint32_t)p.RW + (uint32_t)(x * p.ss + dx);
      // one composite per pixel, or per sample with sample shading (each
      // sample has its own A-buffer at viewSize * layers * sampleID)
      for (int s = 0; s < p.ssn; ++s) {
        const uint32_t eaux = (uint32_t)s * p.P + pixel;
        const size_t abase = (size_t)s * (K == kLoop ? 2 : 1) * p.L * p.P + pixel;
        float4 sum;
        if (K == kRecords) sum = composite_records<L>(p, eaux, abase);
        else if (K == kList || K == kListF32) sum = list_pixel<L, K == kListF32>(p, eaux);
        else if (K == kLoop) sum = composite_loop(p, abase);
        else sum = composite_loop64(p, abase);
        // composite output over the colour target (which already holds the
        // tail-blended opaque + background colour, sample-averaged unless
        // sample shading keeps one per sample)
        float4 c = load_color(p.color, p.color_half != 0, eaux);
        rop_over(c, sum);
        acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
      }
    }
  const float k = 1.0f / (float)(p.ss * p.ss * p.ssn);
  write_out(p, (uint32_t)y * (uint32_t)p.W + (uint32_t)x, make_float4(acc.x * k, acc.y * k, acc.z * k, acc.w * k));
}

// WBOIT composite: oitWeighted.frag.glsl:98-108 with blend
// ONE_MINUS_SRC_ALPHA / SRC_ALPHA (main.cpp:578-588), per sample.
__global__ void __launch_bounds__(256) k_composite_weighted(CompositeParams p) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= p.W || y >= p.H) return;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int dy = 0; dy < p.ss; ++dy)
    for (int dx = 0; dx < p.ss; ++dx) {
      const uint32_t pixel = (uint32_t)(y * p.ss + dy) * (uint32_t)p.RW + (uint32_t)(x * p.ss + dx);
      for (int s = 0; s < p.S; ++s) {
        const size_t o = (size_t)s * p.P + pixel;
        float4 a;
        float rv;
        if (p.weighted_fp32) {
          a = reinterpret_cast<const float4*>(p.accum)[o];
          rv = reinterpret_cast<const float*>(p.reveal)[o];
        } else {
          const uint2 v = reinterpret_cast<const uint2*>(p.accum)[o];
          const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
          const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
          a = make_float4(lo.x, lo.y, hi.x, hi.y);
          rv = __half2float(reinterpret_cast<const __half*>(p.reveal)[o]);
        }
        float4 base = p.has_opaque ? p.opaque_color[o] : p.background;
        const float d = fmaxf(a.w, 1e-5f);
        const float ia = 1.0f - rv;
        base.x = (a.x / d) * ia + base.x * rv;
        base.y = (a.y / d) * ia + base.y * rv;
        base.z = (a.z / d) * ia + base.z * rv;
        base.w = rv * ia + base.w * rv;
        acc.x += base.x; acc.y += base.y; acc.z += base.z; acc.w += base.w;
      }
    }
  const float k = 1.0f / (float)(p.ss * p.ss * p.S);
  write_out(p, (uint32_t)y * (uint32_t)p.W + (uint32_t)x, make_float4(acc.x * k, acc.y * k, acc.z * k, acc.w * k));
}

template <int K>
cudaError_t launch_kind(const CompositeParams& p, cudaStream_t s) {
  const dim3 grid((p.W + 31) / 32, (p.H + 7) / 8), block(256);
  switch (p.L) {
    case 1: k_composite<K, 1><<<grid, block, 0, s>>>(p); break;
    case 2: k_composite<K, 2><<<grid, block, 0, s>>>(p); break;
    case 4: k_composite<K, 4><<<grid, block, 0, s>>>(p); break;
    case 8: k_composite<K, 8><<<grid, block, 0, s>>>(p); break;
    case 16: k_composite<K, 16><<<grid, block, 0, s>>>(p); break;
    case 32: k_composite<K, 32><<<grid, block, 0, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_composite(Alg alg, const CompositeParams& p, cudaStream_t s) {
  const dim3 grid((p.W + 31) / 32, (p.H + 7) / 8), block(256);
  switch (alg) {
    case Alg::Simple:
    case Alg::Spinlock:
    case Alg::Interlock: return launch_kind<kRecords>(p, s);
    case Alg::LinkedList: return p.record_fp32 ? launch_kind<kListF32>(p, s) : launch_kind<kList>(p, s);
    case Alg::Loop: k_composite<kLoop, 1><<<grid, block, 0, s>>>(p); return cudaGetLastError();
    case Alg::Loop64: k_composite<kLoop64, 1><<<grid, block, 0, s>>>(p); return cudaGetLastError();
    case Alg::Weighted: k_composite_weighted<<<grid, block, 0, s>>>(p); return cudaGetLastError();
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace oit
