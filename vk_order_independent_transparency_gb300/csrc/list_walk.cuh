// Linked-list composite of one pixel (oitLinkedList.frag.glsl:106-172) with
// the sort arrays outside registers, so register use (and occupancy) does not
// grow with OIT_LAYERS: a per-thread local array (warp-interleaved in local
// memory, so short lists touch a few L1 lines per warp), or a shared-memory
// column for the first entries.
//
// Semantics, as the reference's composite: the first OIT_LAYERS nodes in list
// order are kept and ordered as bubbleSort orders them
// (oitCompositeDefines.glsl:51-89, swap on >=); every later node goes through
// insertionSortTail (:94-139) and the entry it evicts, or the node itself, is
// tail blended in that order. The kept entries are sorted on insertion as the
// walk goes; bubbleSort's swap-on-equal makes its order of equal depths depend
// on its passes, so when the first OIT_LAYERS nodes hold equal depths they are
// read again and bubbleSort runs itself.
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

// Node loads straight from the pool; colours decoded with the global tables.
template <bool F32>
struct PoolFetch {
  const uint4* __restrict__ pool;
  __device__ __forceinline__ WalkNode operator()(uint32_t off) const { return load_node<F32>(pool, off); }
  __device__ __forceinline__ float4 colour(uint32_t c) const { return node_colour<F32>(pool, c); }
};


// Sort arrays in local memory.
template <bool Mask>
struct WalkArrays {
  static constexpr bool kMask = Mask;
  uint32_t c[kWalkMaxLayers];
  uint32_t d[kWalkMaxLayers];
  uint32_t m[Mask ? kWalkMaxLayers : 1];
  __device__ __forceinline__ uint32_t& C(int i) { return c[i]; }
  __device__ __forceinline__ uint32_t& D(int i) { return d[i]; }
  __device__ __forceinline__ uint32_t& M(int i) { return m[Mask ? i : 0]; }
};

// Sort arrays whose first KS entries live in a shared-memory column of the
// thread (entry i at [i * T], so a warp's lanes always hit distinct banks),
// the rest in local memory (no masks).
template <int KS>
struct SplitArrays {
  static constexpr bool kMask = false;
  uint32_t* sc;
  uint32_t* sd;
  int T;
  uint32_t lc[kWalkMaxLayers - KS], ld[kWalkMaxLayers - KS], lm;
  __device__ __forceinline__ uint32_t& C(int i) { return i < KS ? sc[i * T] : lc[i - KS]; }
  __device__ __forceinline__ uint32_t& D(int i) { return i < KS ? sd[i * T] : ld[i - KS]; }
  __device__ __forceinline__ uint32_t& M(int) { return lm; }
};

struct ListWalk {
  uint32_t head, off, guard;
  int k;
  bool tie;
  float4 tail;
};

// bubbleSort exactly (swap on >=) over the first k nodes in list order, read
// again from the pool.
template <bool F32, class A, class Fetch>
__device__ __noinline__ void walk_bubble(const Fetch& fetch, uint32_t head, uint32_t cap, int k, A& a) {
  constexpr bool Mask = A::kMask;
  uint32_t o = head;
#pragma unroll 1
  for (int i = 0; i < k; ++i) {
    const WalkNode n = fetch(o);
    a.C(i) = n.c;
    a.D(i) = n.d;
    if (Mask) a.M(i) = n.m;
    o = n.next < cap ? n.next : 0u;
  }
#pragma unroll 1
  for (int i = k - 2; i >= 0; --i)
#pragma unroll 1
    for (int j = 0; j <= i; ++j) {
      const uint32_t x = a.D(j), y = a.D(j + 1);
      if (walk_dge(x, y)) {
        uint32_t t = a.C(j);
        a.C(j) = a.C(j + 1);
        a.C(j + 1) = t;
        a.D(j) = y;
        a.D(j + 1) = x;
        if (Mask) {
          t = a.M(j);
          a.M(j) = a.M(j + 1);
          a.M(j + 1) = t;
        }
      }
    }
}

// Consumes node n (the one at w.off). The first OIT_LAYERS nodes are sorted on
// insertion, each placed before equal depths; equal depths are flagged, and on
// reaching OIT_LAYERS nodes (or the end of a shorter list) a flagged array is
// rebuilt by bubbleSort itself. Later nodes go through insertionSortTail.
template <bool F32, class A, class Fetch>
__device__ __forceinline__ void walk_step(ListWalk& w, A& a, const WalkNode& n, const Fetch& fetch,
                                          const uint4* __restrict__ pool, uint32_t cap, int L, int tail) {
  constexpr bool Mask = A::kMask;
  const uint32_t next = n.next < cap ? n.next : 0u;
  if (w.k < L) {
    int pos = w.k;
#pragma unroll 1
    while (pos > 0) {
      const uint32_t dp = a.D(pos - 1);
      if (!walk_dge(dp, n.d)) break;
      w.tie |= !walk_dlt(n.d, dp);  // equal depths
      a.D(pos) = dp;
      a.C(pos) = a.C(pos - 1);
      if (Mask) a.M(pos) = a.M(pos - 1);
      --pos;
    }
    a.D(pos) = n.d;
    a.C(pos) = n.c;
    if (Mask) a.M(pos) = n.m;
    ++w.k;
    w.off = next;
    if (w.tie && (w.k == L || next == 0)) {
      walk_bubble<F32>(fetch, w.head, cap, w.k, a);
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
  if (walk_dlt(n.d, a.D(L - 1))) {
    ev = a.C(L - 1);
    int pos = L - 1;
#pragma unroll 1
    while (pos > 0 && walk_dlt(n.d, a.D(pos - 1))) {
      a.D(pos) = a.D(pos - 1);
      a.C(pos) = a.C(pos - 1);
      if (Mask) a.M(pos) = a.M(pos - 1);
      --pos;
    }
    a.D(pos) = n.d;
    a.C(pos) = n.c;
    if (Mask) a.M(pos) = n.m;
  }
  // the linked list's tail ignores coverage (oitLinkedList.frag.glsl:137-138)
  if (tail) blend_under(w.tail, fetch.colour(ev));
  w.off = next;
}

// Walks the list from `head` and returns the composited colour: kept entries
// front to back (with coverage: per MSAA sample, the entries covering it,
// averaged over the S samples, oitSimple.frag.glsl:142-159), then the tail.
template <bool F32, class A, class Fetch>
__device__ __forceinline__ float4 walk_list_with(const Fetch& fetch, const uint4* __restrict__ pool, uint32_t head,
                                                 uint32_t cap, int L, int tail, int S, A& a) {
  constexpr bool Mask = A::kMask;
  ListWalk w;
  w.head = head < cap ? head : 0u;
  w.off = w.head;
  w.guard = cap;
  w.k = 0;
  w.tie = false;
  w.tail = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
  while (w.off != 0) walk_step<F32>(w, a, fetch(w.off), fetch, pool, cap, L, tail);
  float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!Mask) {
#pragma unroll 1
    for (int i = 0; i < w.k; ++i) blend_under(sum, fetch.colour(a.C(i)));
  } else {
#pragma unroll 1
    for (int s = 0; s < S; ++s) {
      float4 sc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
      for (int i = 0; i < w.k; ++i)
        if ((a.M(i) >> s) & 1u) blend_under(sc, fetch.colour(a.C(i)));
      sum.x += sc.x;
      sum.y += sc.y;
      sum.z += sc.z;
      sum.w += sc.w;
    }
    const float kk = 1.0f / (float)S;
    sum = make_float4(sum.x * kk, sum.y * kk, sum.z * kk, sum.w * kk);
  }
  blend_under(sum, w.tail);
  return sum;
}

template <bool F32, class A>
__device__ __forceinline__ float4 walk_list(const uint4* __restrict__ pool, uint32_t head, uint32_t cap, int L,
                                            int tail, int S, A& a) {
  return walk_list_with<F32>(PoolFetch<F32>{pool}, pool, head, cap, L, tail, S, a);
}

// Sorting networks on (depth, colour) pairs, ascending depth: the 5- and
// 19-comparator networks for 4 and 8 entries (each sorts all 2^K 0-1 inputs,
// so every input). For distinct depths the order equals bubbleSort's.
__device__ __forceinline__ void net_ce(uint32_t& da, uint32_t& ca, uint32_t& db, uint32_t& cb) {
  const bool s = walk_dlt(db, da);
  const uint32_t d0 = da, c0 = ca;
  da = s ? db : da;
  ca = s ? cb : ca;
  db = s ? d0 : db;
  cb = s ? c0 : cb;
}

template <int K>
__device__ __forceinline__ void net_sort(uint32_t (&d)[K], uint32_t (&c)[K]) {
  static_assert(K == 4 || K == 8, "networks for 4 and 8 entries");
#define OIT_CE(a, b) net_ce(d[a], c[a], d[b], c[b])
  if constexpr (K == 4) {
    OIT_CE(0, 1); OIT_CE(2, 3); OIT_CE(0, 2); OIT_CE(1, 3); OIT_CE(1, 2);
  } else {
    OIT_CE(0, 2); OIT_CE(1, 3); OIT_CE(4, 6); OIT_CE(5, 7);
    OIT_CE(0, 4); OIT_CE(1, 5); OIT_CE(2, 6); OIT_CE(3, 7);
    OIT_CE(0, 1); OIT_CE(2, 3); OIT_CE(4, 5); OIT_CE(6, 7);
    OIT_CE(2, 4); OIT_CE(3, 5);
    OIT_CE(1, 4); OIT_CE(3, 6);
    OIT_CE(1, 2); OIT_CE(3, 4); OIT_CE(5, 6);
  }
#undef OIT_CE
}

// Lists of at most K nodes, K <= OIT_LAYERS (all kept, no tail), 1x: the walk
// only appends each node to the thread's shared-memory column (entry i at
// col[i * 32], the columns of a warp's lanes side by side); the entries are
// sorted in registers by the network, which is bubbleSort's order when the
// depths are distinct, and blended from the column. Returns false, with nothing blended, for a list longer than K or
// with equal depths (bubbleSort's order then depends on its passes: the
// caller's full walk runs it).
template <int K>
__device__ __forceinline__ bool walk_list_staged(const uint4* __restrict__ pool, uint32_t head, uint32_t cap,
                                                 uint32_t* sc, uint32_t* sd, float4& sum) {
  constexpr int T = 32;  // the warp's columns: entry i of a lane at [i * 32 + lane]
  uint32_t off = head < cap ? head : 0u;
  int n = 0;
#pragma unroll 1
  while (off != 0) {
    if (n == K) return false;
    const WalkNode nd = load_node<false>(pool, off);
    sc[n * T] = nd.c;
    sd[n * T] = nd.d;
    ++n;
    off = nd.next < cap ? nd.next : 0u;
  }
  {
    uint32_t d[K], c[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      d[i] = i < n ? sd[i * T] : 0x7f800000u;  // +inf after the entries
      c[i] = i < n ? sc[i * T] : 0u;
    }
    net_sort<K>(d, c);
    bool tie = false;
#pragma unroll
    for (int i = 0; i + 1 < K; ++i)
      if (i + 1 < n) tie |= !walk_dlt(d[i], d[i + 1]);
    if (tie) return false;
#pragma unroll
    for (int i = 0; i < K; ++i)
      if (i < n) sc[i * T] = c[i];
  }
  sum = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
  for (int i = 0; i < n; ++i) blend_under(sum, decode_premult(sc[i * T]));
  return true;
}

}  // namespace oitd
