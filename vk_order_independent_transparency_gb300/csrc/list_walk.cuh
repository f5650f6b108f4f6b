// Linked-list composite of one pixel (oitLinkedList.frag.glsl:106-172) as a
// walk that consumes one node per step, with the sort arrays in a per-thread
// local array (warp-interleaved in local memory: short lists touch a few L1
// lines per warp, and occupancy is set by registers, not by OIT_LAYERS).
//
// Semantics, as the reference's composite: the first OIT_LAYERS nodes in list
// order are kept and ordered as bubbleSort orders them
// (oitCompositeDefines.glsl:51-89, swap on >=); every later node goes through
// insertionSortTail (:94-139) and the entry it evicts, or the node itself, is
// tail blended in that order. The kept entries are sorted on insertion;
// bubbleSort's swap-on-equal makes its order of equal depths depend on the
// passes, so when the first OIT_LAYERS nodes hold equal depths they are read
// again and bubbleSort runs itself.
#pragma once

#include "oit_device.cuh"

namespace oitd {

constexpr int kWalkMaxLayers = 32;

__device__ __forceinline__ bool walk_dge(uint32_t a, uint32_t b) { return __uint_as_float(a) >= __uint_as_float(b); }
__device__ __forceinline__ bool walk_dlt(uint32_t a, uint32_t b) { return __uint_as_float(a) < __uint_as_float(b); }

// A list node: packed colour (RGBA8 records) or node index (RGBA32F records,
// whose colour is fetched when blended), depth, coverage mask, next.
struct WalkNode {
  uint32_t c, d, m, next;
};

// F32: 32-byte nodes (float colour, then depth, mask, next); else 16-byte
// nodes {rgba8, depth, mask, next}.
template <bool F32>
__device__ __forceinline__ WalkNode load_node(const uint4* __restrict__ pool, uint32_t off) {
  if (F32) {
    const uint4 n = __ldg(pool + 2 * (size_t)off + 1);
    return WalkNode{off, n.x, n.y, n.z};
  }
  const uint4 n = __ldg(pool + off);
  return WalkNode{n.x, n.y, n.z, n.w};
}

template <bool F32>
__device__ __forceinline__ float4 node_colour(const uint4* __restrict__ pool, uint32_t c) {
  if (F32) {
    const uint4 v = __ldg(pool + 2 * (size_t)c);
    const float a = __uint_as_float(v.w);
    return make_float4(__uint_as_float(v.x) * a, __uint_as_float(v.y) * a, __uint_as_float(v.z) * a, a);
  }
  return decode_premult(c);
}

template <bool Mask>
struct WalkArrays {
  uint32_t c[kWalkMaxLayers];
  uint32_t d[kWalkMaxLayers];
  uint32_t m[Mask ? kWalkMaxLayers : 1];
};

struct ListWalk {
  uint32_t head, off, guard;
  int k;
  bool tie;
  float4 tail;
};

__device__ __forceinline__ void walk_begin(ListWalk& w, uint32_t head, uint32_t cap) {
  w.head = head < cap ? head : 0u;
  w.off = w.head;
  w.guard = cap;
  w.k = 0;
  w.tie = false;
  w.tail = make_float4(0.f, 0.f, 0.f, 0.f);
}

// bubbleSort exactly over the first k nodes in list order.
template <bool F32, bool Mask>
__device__ __noinline__ void walk_bubble(const uint4* __restrict__ pool, uint32_t head, uint32_t cap, int k,
                                         WalkArrays<Mask>& a) {
  uint32_t o = head;
  for (int i = 0; i < k; ++i) {
    const WalkNode n = load_node<F32>(pool, o);
    a.c[i] = n.c;
    a.d[i] = n.d;
    if (Mask) a.m[i] = n.m;
    o = n.next < cap ? n.next : 0u;
  }
  for (int i = k - 2; i >= 0; --i)
    for (int j = 0; j <= i; ++j) {
      const uint32_t x = a.d[j], y = a.d[j + 1];
      if (walk_dge(x, y)) {
        uint32_t t = a.c[j];
        a.c[j] = a.c[j + 1];
        a.c[j + 1] = t;
        a.d[j] = y;
        a.d[j + 1] = x;
        if (Mask) {
          t = a.m[j];
          a.m[j] = a.m[j + 1];
          a.m[j + 1] = t;
        }
      }
    }
}

// Consumes node n (the one at w.off).
template <bool F32, bool Mask>
__device__ __forceinline__ void walk_step(ListWalk& w, WalkArrays<Mask>& a, const WalkNode& n,
                                          const uint4* __restrict__ pool, uint32_t cap, int L, int tail) {
  const uint32_t next = n.next < cap ? n.next : 0u;
  if (w.k < L) {
    int pos = w.k;
    while (pos > 0) {
      const uint32_t dp = a.d[pos - 1];
      if (!walk_dge(dp, n.d)) break;
      w.tie |= !walk_dlt(n.d, dp);  // equal depths
      a.d[pos] = dp;
      a.c[pos] = a.c[pos - 1];
      if (Mask) a.m[pos] = a.m[pos - 1];
      --pos;
    }
    a.d[pos] = n.d;
    a.c[pos] = n.c;
    if (Mask) a.m[pos] = n.m;
    ++w.k;
    w.off = next;
    if (w.tie && (w.k == L || next == 0)) {
      walk_bubble<F32, Mask>(pool, w.head, cap, w.k, a);
      w.tie = false;
    }
    return;
  }
  if (w.guard == 0) {  // bound on a walk (lists built this frame are acyclic)
    w.off = 0;
    return;
  }
  --w.guard;
  uint32_t ev = n.c;
  if (walk_dlt(n.d, a.d[L - 1])) {
    ev = a.c[L - 1];
    int pos = L - 1;
    while (pos > 0 && walk_dlt(n.d, a.d[pos - 1])) {
      a.d[pos] = a.d[pos - 1];
      a.c[pos] = a.c[pos - 1];
      if (Mask) a.m[pos] = a.m[pos - 1];
      --pos;
    }
    a.d[pos] = n.d;
    a.c[pos] = n.c;
    if (Mask) a.m[pos] = n.m;
  }
  // the linked list's tail ignores coverage (oitLinkedList.frag.glsl:137-138)
  if (tail) blend_under(w.tail, node_colour<F32>(pool, ev));
  w.off = next;
}

// Insertion of node n into the first k entries held in registers (static
// indices: K slots, the loop fully unrolled), placed before equal depths as
// the local-array insertion places it; flags equal depths.
template <int K, bool Mask>
__device__ __forceinline__ void insert_reg(uint32_t (&rc)[K], uint32_t (&rd)[K], uint32_t (&rm)[Mask ? K : 1], int k,
                                           const WalkNode& n, bool& tie) {
  bool placed = false;
#pragma unroll
  for (int i = K - 1; i >= 0; --i) {
    if (i <= k && !placed) {
      if (i >= 1 && walk_dge(rd[i - 1], n.d)) {
        tie |= !walk_dlt(n.d, rd[i - 1]);
        rd[i] = rd[i - 1];
        rc[i] = rc[i - 1];
        if (Mask) rm[i] = rm[i - 1];
      } else {
        rd[i] = n.d;
        rc[i] = n.c;
        if (Mask) rm[i] = n.m;
        placed = true;
      }
    }
  }
}

template <bool F32, bool Mask, class Get>
__device__ __forceinline__ float4 blend_kept(const uint4* __restrict__ pool, int k, int S, Get get) {
  float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!Mask) {
    for (int i = 0; i < k; ++i) blend_under(sum, node_colour<F32>(pool, get(i).x));
    return sum;
  }
  for (int s = 0; s < S; ++s) {
    float4 sc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = 0; i < k; ++i) {
      const uint2 e = get(i);
      if ((e.y >> s) & 1u) blend_under(sc, node_colour<F32>(pool, e.x));
    }
    sum.x += sc.x;
    sum.y += sc.y;
    sum.z += sc.z;
    sum.w += sc.w;
  }
  const float kk = 1.0f / (float)S;
  return make_float4(sum.x * kk, sum.y * kk, sum.z * kk, sum.w * kk);
}

// Walks the whole list from `head` and returns the composited colour: kept
// entries front to back (with coverage: per MSAA sample, the entries covering
// it, averaged over the S samples, oitSimple.frag.glsl:142-159), then the tail.
// Lists of at most min(L, K) nodes without equal depths stay in K registers
// per array; longer ones continue in the local arrays `a` (K = 0: always).
template <bool F32, bool Mask, int K = 4>
__device__ __forceinline__ float4 walk_list(const uint4* __restrict__ pool, uint32_t head, uint32_t cap, int L,
                                            int tail, int S, WalkArrays<Mask>& a) {
  constexpr int KR = K > 0 ? K : 1;
  uint32_t rc[KR], rd[KR], rm[Mask ? KR : 1];
  ListWalk w;
  walk_begin(w, head, cap);
  bool local = K == 0;
  while (w.off != 0) {
    const WalkNode n = load_node<F32>(pool, w.off);
    if (!local && w.k < L && w.k < K) {
      insert_reg<KR, Mask>(rc, rd, rm, w.k, n, w.tie);
      ++w.k;
      w.off = n.next < cap ? n.next : 0u;
      if (w.tie && (w.k == L || w.off == 0)) {
        walk_bubble<F32, Mask>(pool, w.head, cap, w.k, a);
        w.tie = false;
        local = true;
      }
      continue;
    }
    if (!local) {
#pragma unroll
      for (int i = 0; i < KR; ++i)
        if (i < w.k) {
          a.c[i] = rc[i];
          a.d[i] = rd[i];
          if (Mask) a.m[i] = rm[i];
        }
      local = true;
    }
    walk_step<F32, Mask>(w, a, n, pool, cap, L, tail);
  }
  float4 sum;
  if (local) {
    sum = blend_kept<F32, Mask>(pool, w.k, S, [&](int i) { return make_uint2(a.c[i], Mask ? a.m[i] : 0u); });
  } else {
    sum = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!Mask) {
#pragma unroll
      for (int i = 0; i < KR; ++i)
        if (i < w.k) blend_under(sum, node_colour<F32>(pool, rc[i]));
    } else {
      for (int s = 0; s < S; ++s) {
        float4 sc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int i = 0; i < KR; ++i)
          if (i < w.k && ((rm[i] >> s) & 1u)) blend_under(sc, node_colour<F32>(pool, rc[i]));
        sum.x += sc.x;
        sum.y += sc.y;
        sum.z += sc.z;
        sum.w += sc.w;
      }
      const float kk = 1.0f / (float)S;
      sum = make_float4(sum.x * kk, sum.y * kk, sum.z * kk, sum.w * kk);
    }
  }
  blend_under(sum, w.tail);
  return sum;
}

}  // namespace oitd
