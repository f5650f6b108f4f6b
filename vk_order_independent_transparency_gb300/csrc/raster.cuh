// Tile rasteriser + per-algorithm A-buffer construction.
//
// One CTA per 16x16 tile, one warp per 8x4 micro-tile, one lane per pixel.
// Each warp walks its tile's triangle list (primitive order, from the bins) in
// chunks of 32: a ballot keeps the triangles whose bbox touches the micro-tile,
// then every kept triangle is rasterised against the warp's 32 pixels (and
// their MSAA samples). A covered pixel's lane runs the algorithm's fragment
// body (the COLOR/DEPTH shader of the reference) on that pixel's state, so
// every pixel sees its fragments in primitive order -- the order the
// reference's hardware blender guarantees for tail blending and the order
// ordered interlock guarantees for its critical section. Per-pixel k-buffers
// live in shared memory or registers; the A-buffer, aux images and the
// tail-blended colour target are written to HBM once, at the end.
#pragma once

#include <cuda_fp16.h>

#include <algorithm>

#include "oit_device.cuh"

namespace oitd {

using oit::RasterParams;

constexpr uint32_t kFull = 0xffffffffu;
constexpr unsigned long long kEmpty64 = 0xFFFFFFFFFFFFFFFFull;

// A transparent fragment as the fragment shaders see it.
struct Frag {
  uint32_t packed;  // packUnorm4x8(unPremultLinearToSRGB(shading))
  uint32_t depth;   // floatBitsToUint(gl_FragCoord.z)
  uint32_t cover;   // samples covered after early depth (gl_SampleMaskIn with post_depth_coverage)
  float r, g, b, a; // shading(): linear, unpremultiplied
  float view_z;     // Interpolants::depth
};

template <int S>
struct PixelTargets {
  uint32_t depth[S];  // opaque depth per sample
  float4 col[S];      // colour target per sample (premultiplied linear)

  __device__ __forceinline__ void tail(const float4& src, uint32_t cover) {
#pragma unroll
    for (int s = 0; s < S; ++s)
      if (cover & (1u << s)) rop_over(col[s], src);
  }
};

__device__ __forceinline__ float4 premult(float r, float g, float b, float a) {
  return make_float4(r * a, g * a, b * a, a);
}

// ---------------------------------------------------------------------------
// Policies. Each provides: kPasses, kShade (needs colour), kViewZ,
// smem_bytes_per_warp(L, coverage), init(p, smem, lane, sample, pixel),
// fragment(pass, f, node, targets), flush(p, valid). `sample` is the lane's
// sample with sample shading (each sample has its own A-buffer) and 0 otherwise.
// fragment() runs on the pixel's owner lane only, once per fragment, in
// primitive order.
// ---------------------------------------------------------------------------

// oitSimple.frag.glsl:50-91
template <int S>
struct SimplePolicy {
  static constexpr bool kNodes = false;
  static constexpr int kPasses = 1;
  // resident warps per SM with one coverage sample per lane (sets the register
  // budget: 36 -> 56 registers, spill-free or nearly; 32 -> 64 where 56 spills)
  static constexpr int kWarpsPerSM = 36;
  static constexpr bool kViewZ = false;
  static __host__ __device__ size_t smem_bytes_per_warp(int, int, int = 0) { return 0; }
  uint32_t count;
  uint32_t eaux;
  size_t abase;  // listPos = viewSize * OIT_LAYERS * sampleID + pixel (oitSimple.frag.glsl:60)
  __device__ void init(const RasterParams& p, void*, int, int sample, uint32_t pixel) {
    count = 0;
    eaux = (uint32_t)sample * p.P + pixel;
    abase = (size_t)sample * p.L * p.P + pixel;
  }
  __device__ __forceinline__ void fragment(const RasterParams& p, int, const Frag& f, uint32_t, PixelTargets<S>& tg) {
    const uint32_t old = count++;
    if (old < (uint32_t)p.L) {
      const size_t r = abase + (size_t)old * p.P;
      if (p.coverage) {
        reinterpret_cast<uint4*>(p.abuf)[r] = make_uint4(f.packed, f.depth, f.cover, 0u);
      } else {
        reinterpret_cast<uint2*>(p.abuf)[r] = make_uint2(f.packed, f.depth);
      }
    } else if (p.tail) {
      tg.tail(premult(f.r, f.g, f.b, f.a), f.cover);
    }
  }
  __device__ void flush(const RasterParams& p, bool valid) {
    if (valid) p.aux[eaux] = count;
  }
};

// oitLinkedList.frag.glsl:51-85. The node counter is a global atomic,
// aggregated per warp: one atomicAdd per batch of queued fragments hands out
// consecutive node indices in queue (primitive, then pixel) order.
template <int S>
struct LinkedListPolicy {
  static constexpr int kPasses = 1;
  // resident warps per SM with one coverage sample per lane (sets the register
  // budget: 36 -> 56 registers, spill-free or nearly; 32 -> 64 where 56 spills)
  static constexpr int kWarpsPerSM = 36;
  static constexpr bool kViewZ = false;
  static constexpr bool kNodes = true;
  static __host__ __device__ size_t smem_bytes_per_warp(int, int, int = 0) { return 0; }
  uint32_t head;
  uint32_t eaux;
  __device__ void init(const RasterParams& p, void*, int, int sample, uint32_t pixel) {
    head = 0;
    eaux = (uint32_t)sample * p.P + pixel;
  }
  // node: the index the batched counter allocation gave this fragment
  // (imageAtomicAdd(imgCounter) + 1, oitLinkedList.frag.glsl:55).
  __device__ __forceinline__ void fragment(const RasterParams& p, int, const Frag& f, uint32_t node,
                                           PixelTargets<S>& tg) {
    if (node >= p.capacity) {
      if (p.tail) tg.tail(premult(f.r, f.g, f.b, f.a), f.cover);
      return;
    }
    if (p.record_fp32) {
      // RGBA32F node: linear unpremultiplied colour, then depth, mask, next
      uint4* n = reinterpret_cast<uint4*>(p.abuf) + 2 * (size_t)node;
      n[0] = make_uint4(__float_as_uint(f.r), __float_as_uint(f.g), __float_as_uint(f.b), __float_as_uint(f.a));
      n[1] = make_uint4(f.depth, p.coverage ? f.cover : 0u, head, 0u);
    } else {
      reinterpret_cast<uint4*>(p.abuf)[node] = make_uint4(f.packed, f.depth, p.coverage ? f.cover : 0u, head);
    }
    head = node;
  }
  __device__ void flush(const RasterParams& p, bool valid) {
    if (valid) p.aux[eaux] = head;
  }
};

// oitLoop64.frag.glsl:65-141. The per-pixel k-buffer of 64-bit keys
// (depth << 32 | rgba8) lives in shared memory, [layer][lane] per warp; the
// atomicMin insertion loop runs on it in primitive order.
template <int S>
struct Loop64Policy {
  static constexpr bool kNodes = false;
  static constexpr int kPasses = 1;
  // resident warps per SM with one coverage sample per lane (sets the register
  // budget: 36 -> 56 registers, spill-free or nearly; 32 -> 64 where 56 spills)
  static constexpr int kWarpsPerSM = 36;
  static constexpr bool kViewZ = false;
  // keys, plus a float4 colour per slot with RGBA32F records
  static __host__ __device__ size_t smem_bytes_per_warp(int L, int, int fp32 = 0) {
    return (size_t)L * 32 * (fp32 ? 24 : 8);
  }
  unsigned long long* kb;
  float4* pay;  // RGBA32F payload moving with its key, or null
  int lane;
  size_t abase;
  __device__ void init(const RasterParams& p, void* smem, int, int sample, uint32_t pixel) {
    lane = threadIdx.x & 31;
    abase = (size_t)sample * p.L * p.P + pixel;
    kb = reinterpret_cast<unsigned long long*>(smem);
    pay = p.record_fp32 ? reinterpret_cast<float4*>(kb + p.L * 32) : nullptr;
    for (int i = 0; i < p.L; ++i) kb[i * 32 + lane] = kEmpty64;
  }
  __device__ __forceinline__ void fragment(const RasterParams& p, int, const Frag& f, uint32_t, PixelTargets<S>& tg) {
    const int L = p.L;
    unsigned long long zcur = ((unsigned long long)f.depth << 32) | f.packed;
    float4 pcur = make_float4(f.r, f.g, f.b, f.a);
    bool evict = true;
    if (!(zcur > kb[(L - 1) * 32 + lane])) {
      int i = (zcur > kb[(L / 2) * 32 + lane]) ? (L / 2) : 0;
      for (; i < L; ++i) {
        const unsigned long long ztest = kb[i * 32 + lane];
        if (zcur < ztest) {
          kb[i * 32 + lane] = zcur;
          if (pay) {
            const float4 t = pay[i * 32 + lane];
            pay[i * 32 + lane] = pcur;
            pcur = t;
          }
        }
        if (ztest == kEmpty64) {
          evict = false;
          break;
        }
        zcur = ztest > zcur ? ztest : zcur;
      }
    }
    if (evict && p.tail) tg.tail(pay ? premult(pcur.x, pcur.y, pcur.z, pcur.w) : decode_premult((uint32_t)zcur), f.cover);
  }
  __device__ void flush(const RasterParams& p, bool valid) {
    if (!valid) return;
    unsigned long long* ab = reinterpret_cast<unsigned long long*>(p.abuf);
    for (int i = 0; i < p.L; ++i) ab[abase + (size_t)i * p.P] = kb[i * 32 + lane];
    if (pay) {
      // payload block after the keys of every sample: [sample][layer][pixel] float4
      float4* pb = reinterpret_cast<float4*>(ab + (size_t)p.ssn * p.L * p.P);
      for (int i = 0; i < p.L; ++i) pb[abase + (size_t)i * p.P] = pay[i * 32 + lane];
    }
  }
};

// oitLoop.frag.glsl:57-100 (DEPTH pass 0) and 120-173 (COLOR pass 1). Both
// passes walk the same triangle list; the sorted depths stay in shared memory
// between them.
template <int S>
struct LoopPolicy {
  static constexpr bool kNodes = false;
  static constexpr int kPasses = 2;
  // resident warps per SM with one coverage sample per lane (sets the register
  // budget: 36 -> 56 registers, spill-free or nearly; 32 -> 64 where 56 spills)
  static constexpr int kWarpsPerSM = 32;
  static constexpr bool kViewZ = false;
  static __host__ __device__ size_t smem_bytes_per_warp(int L, int, int = 0) { return (size_t)L * 32 * 8; }
  uint32_t* dep;
  uint32_t* col;
  int lane;
  size_t abase;  // viewSize * OIT_LAYERS * 2 * sampleID + pixel (oitLoop.frag.glsl:231)
  __device__ void init(const RasterParams& p, void* smem, int, int sample, uint32_t pixel) {
    lane = threadIdx.x & 31;
    abase = (size_t)sample * 2 * p.L * p.P + pixel;
    dep = reinterpret_cast<uint32_t*>(smem);
    col = dep + p.L * 32;
    for (int i = 0; i < p.L; ++i) {
      dep[i * 32 + lane] = 0xFFFFFFFFu;
      col[i * 32 + lane] = 0u;
    }
  }
  __device__ __forceinline__ void fragment(const RasterParams& p, int pass, const Frag& f, uint32_t,
                                           PixelTargets<S>& tg) {
    const int L = p.L;
    uint32_t zcur = f.depth;
    if (pass == 0) {
      if (zcur > dep[(L - 1) * 32 + lane]) return;
      int i = (zcur > dep[(L / 2) * 32 + lane]) ? (L / 2) : 0;
      for (; i < L; ++i) {
        const uint32_t ztest = dep[i * 32 + lane];
        if (zcur < ztest) dep[i * 32 + lane] = zcur;
        if (ztest == 0xFFFFFFFFu || ztest == zcur) break;
        zcur = ztest > zcur ? ztest : zcur;
      }
    } else {
      if (dep[(L - 1) * 32 + lane] < zcur) {
        if (p.tail) tg.tail(premult(f.r, f.g, f.b, f.a), f.cover);
        return;
      }
      int start = 0, end = L - 1;
      while (start < end) {
        const int mid = (start + end) / 2;
        if (dep[mid * 32 + lane] < zcur) start = mid + 1; else end = mid;
      }
      col[start * 32 + lane] = f.packed;
    }
  }
  __device__ void flush(const RasterParams& p, bool valid) {
    if (!valid) return;
    for (int i = 0; i < p.L; ++i) {
      p.abuf[abase + (size_t)i * p.P] = dep[i * 32 + lane];
      p.abuf[abase + (size_t)(p.L + i) * p.P] = col[i * 32 + lane];
    }
  }
};

// oitSpinlock.frag.glsl:49-129 / oitInterlock.frag.glsl:90-152. The pixel's
// owner lane is its critical section: no lock is needed because no other
// thread ever touches the pixel, and fragments arrive in primitive order.
template <int S>
struct LockPolicy {
  static constexpr bool kNodes = false;
  static constexpr int kPasses = 1;
  // resident warps per SM with one coverage sample per lane (sets the register
  // budget: 36 -> 56 registers, spill-free or nearly; 32 -> 64 where 56 spills)
  static constexpr int kWarpsPerSM = 36;
  static constexpr bool kViewZ = false;
  static __host__ __device__ size_t smem_bytes_per_warp(int L, int coverage, int = 0) {
    return (size_t)L * 32 * (coverage ? 16 : 8);
  }
  uint32_t count, auxdepth;
  uint32_t* rec;  // [layer][lane] x words
  int lane, words;
  uint32_t eaux;
  size_t abase;
  __device__ void init(const RasterParams& p, void* smem, int, int sample, uint32_t pixel) {
    lane = threadIdx.x & 31;
    eaux = (uint32_t)sample * p.P + pixel;
    abase = (size_t)sample * p.L * p.P + pixel;
    words = p.coverage ? 4 : 2;
    rec = reinterpret_cast<uint32_t*>(smem);
    count = 0;
    auxdepth = 0xFFFFFFFFu;
  }
  __device__ __forceinline__ uint32_t* slot(int i) const { return rec + ((size_t)i * 32 + lane) * words; }
  __device__ __forceinline__ void fragment(const RasterParams& p, int, const Frag& f, uint32_t, PixelTargets<S>& tg) {
    const int L = p.L;
    float4 out = premult(f.r, f.g, f.b, f.a);
    if (f.depth <= auxdepth) {
      const uint32_t old = count++;
      if (old < (uint32_t)L) {
        uint32_t* r = slot((int)old);
        r[0] = f.packed;
        r[1] = f.depth;
        if (words == 4) {
          r[2] = f.cover;
          r[3] = 0u;
        }
        out = make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        int furthest = 0;
        uint32_t maxDepth = 0;
        for (int i = 0; i < L; ++i) {
          const uint32_t d = slot(i)[1];
          if (d > maxDepth) {
            maxDepth = d;
            furthest = i;
          }
        }
        if (maxDepth > f.depth) {
          uint32_t* r = slot(furthest);
          out = decode_premult(r[0]);
          r[0] = f.packed;
          r[1] = f.depth;
          if (words == 4) {
            r[2] = f.cover;
            r[3] = 0u;
          }
          auxdepth = maxDepth;
        }
      }
    }
    if (p.tail) tg.tail(out, f.cover);
  }
  __device__ void flush(const RasterParams& p, bool valid) {
    if (!valid) return;
    p.aux[eaux] = count;
    p.auxdepth[eaux] = auxdepth;
    const int n = count < (uint32_t)p.L ? (int)count : p.L;
    for (int i = 0; i < n; ++i) {
      const uint32_t* r = slot(i);
      const size_t o = abase + (size_t)i * p.P;
      if (words == 4) {
        reinterpret_cast<uint4*>(p.abuf)[o] = make_uint4(r[0], r[1], r[2], r[3]);
      } else {
        reinterpret_cast<uint2*>(p.abuf)[o] = make_uint2(r[0], r[1]);
      }
    }
  }
};

// oitWeighted.frag.glsl:53-79 with the blend state of main.cpp:559-577.
// FP16 mode rounds the accumulators to half after every blend, as an
// RGBA16F/R16F render target does.
template <int S>
struct WeightedPolicy {
  static constexpr bool kNodes = false;
  static constexpr int kPasses = 1;
  // resident warps per SM with one coverage sample per lane: 36 (56
  // registers, a few spills) measured faster than 32 at 3840x2160 (6.84 vs 6.89 ms)
  static constexpr int kWarpsPerSM = 36;
  static constexpr bool kViewZ = true;
  static __host__ __device__ size_t smem_bytes_per_warp(int, int, int = 0) { return 0; }
  float4 acc[S];
  float rev[S];
  uint32_t px_;
  __device__ void init(const RasterParams&, void*, int, int, uint32_t pixel) {
    px_ = pixel;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      acc[s] = make_float4(0.f, 0.f, 0.f, 0.f);
      rev[s] = 1.0f;
    }
  }
  static __device__ __forceinline__ float h(float x) { return __half2float(__float2half_rn(x)); }
  __device__ __forceinline__ void fragment(const RasterParams& p, int, const Frag& f, uint32_t, PixelTargets<S>&) {
    const float4 c = premult(f.r, f.g, f.b, f.a);
    const float depthZ = -f.view_z * 10.0f;
    const float x = depthZ / 200.0f;
    const float x2 = x * x;
    float distWeight = 0.03f / (1e-5f + x2 * x2);
    distWeight = fminf(fmaxf(distWeight, 1e-2f), 3e3f);
    float aw = fminf(1.0f, fmaxf(fmaxf(c.x, c.y), fmaxf(c.z, c.w)) * 40.0f + 0.01f);
    aw *= aw;
    const float w = aw * distWeight;
    const float4 src = make_float4(c.x * w, c.y * w, c.z * w, c.w * w);
    const bool fp16 = !p.weighted_fp32;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      if (!(f.cover & (1u << s))) continue;
      if (fp16) {
        acc[s].x = h(acc[s].x + h(src.x));
        acc[s].y = h(acc[s].y + h(src.y));
        acc[s].z = h(acc[s].z + h(src.z));
        acc[s].w = h(acc[s].w + h(src.w));
        rev[s] = h(rev[s] * (1.0f - h(c.w)));
      } else {
        acc[s].x += src.x;
        acc[s].y += src.y;
        acc[s].z += src.z;
        acc[s].w += src.w;
        rev[s] *= (1.0f - c.w);
      }
    }
  }
  __device__ void flush(const RasterParams& p, bool valid) {
    if (!valid) return;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const size_t o = (size_t)s * p.P + px_;
      if (p.weighted_fp32) {
        reinterpret_cast<float4*>(p.accum)[o] = acc[s];
        reinterpret_cast<float*>(p.reveal)[o] = rev[s];
      } else {
        __half2 lo = __floats2half2_rn(acc[s].x, acc[s].y);
        __half2 hi = __floats2half2_rn(acc[s].z, acc[s].w);
        uint2 v;
        v.x = *reinterpret_cast<uint32_t*>(&lo);
        v.y = *reinterpret_cast<uint32_t*>(&hi);
        reinterpret_cast<uint2*>(p.accum)[o] = v;
        reinterpret_cast<__half*>(p.reveal)[o] = __float2half_rn(rev[s]);
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Triangle-list walk shared by the transparent and opaque kernels.
// ---------------------------------------------------------------------------
// A warp's piece of a 16x16 tile. Without sample shading (SSN = 1) a warp
// owns an 8x4 micro-tile, one lane per pixel, and a CTA of 8 warps covers the
// tile. With sample shading every sample has its own A-buffer, so a lane owns
// one sample: a warp covers 4x2 pixels x 4 samples or 2x2 pixels x 8 samples
// and SSN CTAs cover the tile.
struct WarpTile {
  int lane, px, py, rx0, ry0, rx1, ry1;
  int mt;      // the warp's micro-tile (or sample group) within the tile
  int sample;  // the lane's sample with sample shading, else 0
  bool valid;
  uint32_t pixel;
};

template <int SSN>
struct LaneMap {
  static constexpr int kPix = 32 / SSN;                  // pixels per warp
  static constexpr int kW = SSN == 1 ? 8 : (SSN == 4 ? 4 : 2);
  static constexpr int kH = kPix / kW;
  __device__ static int pix(int lane) { return lane % kPix; }
  __device__ static int sample(int lane) { return lane / kPix; }
};

// cta: the CTA's index within its view's grid.
template <int SSN>
__device__ __forceinline__ WarpTile warp_tile(const RasterParams& p, int cta) {
  using M = LaneMap<SSN>;
  WarpTile w;
  const int warp = threadIdx.x >> 5;
  w.lane = threadIdx.x & 31;
  const int gw = cta * (int)(blockDim.x >> 5) + warp;   // warp within the pass
  const int tile = gw / (oit::kWarpsPerTile * SSN);
  const int mt = gw % (oit::kWarpsPerTile * SSN);           // micro-tile within the tile
  w.mt = mt;
  const int tx = tile % p.tiles_x, ty = tile / p.tiles_x;
  w.rx0 = tx * 16 + (mt % (16 / M::kW)) * M::kW;
  w.ry0 = ty * 16 + (mt / (16 / M::kW)) * M::kH;
  w.rx1 = w.rx0 + M::kW - 1;
  w.ry1 = w.ry0 + M::kH - 1;
  const int pix = M::pix(w.lane);
  w.sample = M::sample(w.lane);
  w.px = w.rx0 + pix % M::kW;
  w.py = w.ry0 + pix / M::kW;
  w.valid = w.px < p.RW && w.py < p.RH;
  w.pixel = w.valid ? (uint32_t)w.py * (uint32_t)p.RW + (uint32_t)w.px : 0u;
  return w;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__device__ __forceinline__ bool bbox_hits(uint2 bb, const WarpTile& w) {
  const int bx0 = bb.x & 0xFFFF, by0 = bb.x >> 16, bx1 = bb.y & 0xFFFF, by1 = (bb.y >> 16) & 0x7FFF;
  return !(bx1 < w.rx0 || bx0 > w.rx1 || by1 < w.ry0 || by0 > w.ry1);
}

// Setup records a warp stages at once: every hit of a 32-entry chunk of the
// tile list. (16 slots, with a second round for chunks holding more hits,
// left shared memory for more resident warps at Loop64's larger k-buffers:
// the 1080p Loop64 raster 0.346 -> 0.337 ms, but the 64-view batch 19.15 ->
// 20.6 ms in one run.)
constexpr int kStageSlots = 32;

// Walks [beg, end) of the tile list in primitive order, 32 entries at a time:
// the lanes test their triangle against the warp's micro-tile, the hits copy
// their setup records into the warp's shared-memory stage in parallel
// (cp.async) with their triangle ids and bboxes, then chunk(nh) processes
// stage slots 0..nh-1, which are in list order. chunk is warp-uniform.
// Mask (8x4 micro-tiles, one lane per pixel): the test is the micro-tile's bit
// in the pair's sorted key (the binning wrote the bbox's micro-tile overlap
// there), so only hits gather their bbox; else the bbox itself is tested.
// List entries of triangles >= limit are skipped (the second half of a
// near-clipped triangle t, record num_tris + t, counts as triangle t). With
// `ident` (an overflowed draw's unbinned triangles) entry i of [beg, end) is
// half i & 1 of triangle i >> 1, tested by its bbox (a second half only when
// the first's bbox says it exists).
template <bool Mask, class Chunk>
__device__ __forceinline__ void walk_tile(const RasterParams& p, const WarpTile& w, TriSetup* stage,
                                          uint32_t* stage_t, uint2* stage_bb, uint32_t beg, uint32_t end,
                                          bool ident, uint32_t limit, Chunk&& chunk) {
  const TriSetup* __restrict__ setup = reinterpret_cast<const TriSetup*>(p.setup);
  const uint32_t lt = (1u << w.lane) - 1u;
  const uint32_t mbit = 1u << (oit::kMaskShift + (Mask ? w.mt : 0));
  const bool use_mask = Mask && !ident;
  uint32_t t_next = 0;
  bool h_next = false;
  uint2 bb_next = make_uint2(0xFFFFFFFFu, 0u);  // empty bbox
  auto orig = [&](uint32_t t) { return t >= p.num_tris ? t - p.num_tris : t; };
  auto fetch = [&](uint32_t i) {
    t_next = ident ? ((i & 1u) ? p.num_tris + (i >> 1) : (i >> 1)) : __ldg(&p.tile_tris[i]);
    if (use_mask) h_next = (__ldg(&p.tile_keys[i]) & mbit) != 0u && orig(t_next) < limit;
  };
  // a second half exists when its first half's bbox says so
  auto fetch_bb = [&](uint32_t i) {
    if (ident && (i & 1u) && !(__ldg(&p.bbox[i >> 1]).y >> 31)) return make_uint2(0xFFFFFFFFu, 0u);
    return __ldg(&p.bbox[t_next]);
  };
  if (beg + w.lane < end) {
    fetch(beg + w.lane);
    if (!use_mask || h_next) bb_next = fetch_bb(beg + w.lane);
  }
  for (uint32_t base = beg; base < end; base += 32) {
    const uint32_t t = t_next;
    const uint2 bb = bb_next;
    const bool hit = (base + w.lane < end) && (use_mask ? h_next : (bbox_hits(bb, w) && orig(t) < limit));
    const uint32_t nb = base + 32;
    const bool more = nb + w.lane < end;
    if (more) fetch(nb + w.lane);
    else h_next = false;
    const uint32_t m = __ballot_sync(kFull, hit);
    const int rank = __popc(m & lt);
    auto stage_hit = [&](int slot) {
      const int4* src = reinterpret_cast<const int4*>(setup + t);
      int4* dst = reinterpret_cast<int4*>(stage + slot);
#pragma unroll
      for (int k = 0; k < 6; ++k) cp_async16(dst + k, src + k);
      stage_t[slot] = t;
      stage_bb[slot] = bb;
    };
    if (hit) stage_hit(rank);
    bb_next = more && (!use_mask || h_next) ? fetch_bb(nb + w.lane) : make_uint2(0xFFFFFFFFu, 0u);
    cp_async_wait_all();
    __syncwarp();
    if (m) chunk(__popc(m));
    __syncwarp();
  }
}

// Triangles of the draw binned whole: all of them, or after a bin overflow
// those before the first triangle whose pairs reach past the capacity (pairs
// are emitted in triangle order). Warp-uniform.
__device__ __forceinline__ uint32_t binned_triangles(const RasterParams& p) {
  if (!p.pair_total || *p.pair_total <= p.pair_capacity) return 0xFFFFFFFFu;
  uint32_t lo = 0, hi = p.num_tris;  // first t with pair_offset[t] + pair_count[t] > capacity
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&p.pair_offset[mid]) + __ldg(&p.pair_count[mid]) > p.pair_capacity) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// The pass's walk: the tile list (triangles binned whole), then, after a bin
// overflow, the unbinned triangles of the pass by bbox; primitive order is
// kept because every binned triangle precedes every unbinned one.
template <bool Mask, class Chunk>
__device__ __forceinline__ void walk_pass(const RasterParams& p, const WarpTile& w, TriSetup* stage,
                                          uint32_t* stage_t, uint2* stage_bb, uint32_t beg, uint32_t end,
                                          Chunk&& chunk) {
  const uint32_t cut = binned_triangles(p);
  const bool rest = cut < p.pass_end;
  const uint32_t nph = rest ? 2u : 1u;
#pragma unroll 1
  for (uint32_t ph = 0; ph < nph; ++ph) {
    const bool ident = ph == 1;
    walk_tile<Mask>(p, w, stage, stage_t, stage_bb, ident ? 2u * max(cut, p.pass_first) : beg,
                    ident ? 2u * p.pass_end : end, ident, ident ? 0xFFFFFFFFu : cut, chunk);
  }
}

__device__ __forceinline__ bool lane_in_bbox(uint2 bb, const WarpTile& w) {
  return w.valid && w.px >= (int)(bb.x & 0xFFFF) && w.px <= (int)(bb.y & 0xFFFF) && w.py >= (int)(bb.x >> 16) &&
         w.py <= (int)((bb.y >> 16) & 0x7FFF);
}

// Per-warp fragment queue: coverage appends (stage slot, lane, coverage,
// depth) in primitive-then-lane order; shading runs one queued fragment per
// lane once a staged chunk is covered (the setup records it reads are then
// replaced); when the queue is full, and at the end, each lane feeds its own
// pixel's fragments, in queue order, to the algorithm (feeding a full queue
// rather than each chunk's fragments: fewer passes over the owner bytes and
// linked-list node allocations of up to kQueue nodes). vz holds the
// view-space z (WBOIT, which feeds per chunk) or, for every other algorithm,
// the fragment's alpha.
constexpr int kQueue = 64;
struct FragQueue {
  uint32_t depth[kQueue];
  uint32_t packed[kQueue];
  float r[kQueue], g[kQueue], b[kQueue], vz[kQueue];
  unsigned char tri[kQueue], lane[kQueue], cover[kQueue], pad[kQueue];
};
// per warp: kStageSlots staged records, their triangle ids and bboxes, the queue, and
// the per-hit pixel ranges of the coverage enumeration
struct HitRanges {
  // per hit: prefix (bits 0-10, exclusive prefix of the pixel counts), x and y
  // of bbox ∩ micro-tile relative to the micro-tile (bits 11-13, 14-15), its
  // width (bits 16-19) and ceil(256 / width) (bits 20-28)
  uint32_t packed[32];
};
constexpr size_t kWarpStageBytes = kStageSlots * (sizeof(TriSetup) + sizeof(uint32_t) + sizeof(uint2)) +
                                   sizeof(FragQueue) + sizeof(HitRanges);

// ---------------------------------------------------------------------------
// Transparent COLOR (+DEPTH) pass.
// ---------------------------------------------------------------------------
// S: samples each lane evaluates (MSAA coverage); SSN: samples mapped to
// lanes (sample shading, S = 1 then).
// The warps of a tile work independently (each walks the tile's list for its
// own micro-tile), so a CTA holds kRasterWarpsPerBlock of them: a CTA's
// resources are released when its slowest warp is done, and micro-tiles of
// one tile differ in work (2 warps per CTA: the 64-view batch 5.6% faster
// than 8; Loop64 k-buffers at large OIT_LAYERS pack shared memory better).
using oit::kRasterWarpsPerBlock;
// Policy::kWarpsPerSM resident warps per SM for one coverage sample per lane
// (36 at 56 registers: the 64-view batch 19.28 -> 18.96 ms against 32 at 64;
// shared memory still limits Loop64 and Loop32 at large OIT_LAYERS), 24 for
// MSAA lanes, whose per-sample state needs more.
template <template <int> class Policy, int S, int SSN>
__device__ __forceinline__ void raster_transparent_body(const RasterParams& p, int cta) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using Pol = Policy<S>;
  using M = LaneMap<SSN>;
  const int warp = threadIdx.x >> 5;
  const WarpTile w = warp_tile<SSN>(p, cta);
  const uint32_t elem = (uint32_t)w.sample * p.P + w.pixel;  // this lane's sample of the pixel
  unsigned char* wbase = smem_raw + (size_t)warp * kWarpStageBytes;
  TriSetup* stage = reinterpret_cast<TriSetup*>(wbase);
  uint32_t* stage_t = reinterpret_cast<uint32_t*>(wbase + kStageSlots * sizeof(TriSetup));
  uint2* stage_bb = reinterpret_cast<uint2*>(wbase + kStageSlots * (sizeof(TriSetup) + sizeof(uint32_t)));
  FragQueue* q =
      reinterpret_cast<FragQueue*>(wbase + kStageSlots * (sizeof(TriSetup) + sizeof(uint32_t) + sizeof(uint2)));
  HitRanges* hr = reinterpret_cast<HitRanges*>(
      wbase + kStageSlots * (sizeof(TriSetup) + sizeof(uint32_t) + sizeof(uint2)) + sizeof(FragQueue));
  unsigned char* pol_smem = smem_raw + (size_t)(blockDim.x >> 5) * kWarpStageBytes +
                            (size_t)warp * Pol::smem_bytes_per_warp(p.L, p.coverage, p.record_fp32);

  PixelTargets<S> tg;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const size_t o = (size_t)(SSN > 1 ? w.sample : s) * p.P + w.pixel;
    if (p.has_opaque && w.valid) {
      tg.depth[s] = p.depth[o];
      tg.col[s] = p.opaque_color[o];
    } else {
      tg.depth[s] = 0x3F800000u;  // 1.0f
      tg.col[s] = p.background;
    }
  }
  Pol pol;
  pol.init(p, pol_smem, w.lane, w.sample, w.pixel);

  const int tile = (int)((cta * (blockDim.x >> 5) + warp) / (oit::kWarpsPerTile * SSN)) + p.tile_offset;
  const uint32_t beg = p.tile_begin[tile], end = p.tile_end[tile];
  const TriPersp* __restrict__ persp = reinterpret_cast<const TriPersp*>(p.persp);
  const uint32_t lt = (1u << w.lane) - 1u;
  uint32_t nfrag = 0;  // warp-uniform
  uint32_t mine = 0;   // fragments delivered to this lane's pixel
  int qn = 0;          // warp-uniform: queued fragments
  int qs = 0;          // warp-uniform: queued fragments already shaded
  const uint32_t lane_bytes = (uint32_t)w.lane * 0x01010101u;

  for (int pass = 0; pass < Pol::kPasses; ++pass) {
    const bool shading = Pol::kPasses == 1 || pass == Pol::kPasses - 1;

    // Shades queue entries [qs, qn): their setup records are still staged.
    auto shade_pending = [&]() {
      if (!shading || qs == qn) {
        qs = qn;
        return;
      }
      __syncwarp();
      for (int j = qs + w.lane; j < qn; j += 32) {
        const TriSetup& T = stage[q->tri[j]];
        const int l = q->lane[j];
        // shading point: the pixel centre, or the lane's sample with sample shading
        const int pl = M::pix(l);
        const int2 sp = SSN > 1 ? sample_pos<SSN>(M::sample(l)) : make_int2(128, 128);
        const int sx = (w.rx0 + pl % M::kW) * 256 + sp.x, sy = (w.ry0 + pl / M::kW) * 256 + sp.y;
        const TriPersp* P = Pol::kViewZ ? persp + stage_t[q->tri[j]] : nullptr;
        const int4 a = T.xy01, b = T.xy2f;
        Shade sh;
        if (b.z & kFlagSmall) sh = shade(T, edges_at<int>(a, b, sx, sy), P);
        else sh = shade(T, edges_at<long long>(a, b, sx, sy), P);
        q->packed[j] = pack_rgba8(sh, (uint32_t)(b.z >> 8) & 255u);
        q->r[j] = sh.r;
        q->g[j] = sh.g;
        q->b[j] = sh.b;
        q->vz[j] = Pol::kViewZ ? sh.view_z : __int_as_float(b.w);  // view z, or alpha
      }
      qs = qn;
      __syncwarp();
    };

    // Feeds the queue to the algorithm (after shading what is left).
    auto flush = [&]() {
      if (qn == 0) return;
      shade_pending();
      uint32_t node0 = 0;
      if (Pol::kNodes && shading) {
        if (w.lane == 0) node0 = atomicAdd(p.counter, (uint32_t)qn);
        node0 = __shfl_sync(kFull, node0, 0);
      }
      // this lane's entries: scan the owner byte of every queued fragment
      unsigned long long mm = 0;
      const uint32_t* lanes = reinterpret_cast<const uint32_t*>(q->lane);
      for (int wi = 0; wi * 4 < qn; ++wi) {
        const uint32_t eq = __vcmpeq4(lanes[wi], lane_bytes);  // 0xff per matching byte
        const uint32_t bits = ((eq >> 7) & 1u) | ((eq >> 14) & 2u) | ((eq >> 21) & 4u) | ((eq >> 28) & 8u);
        mm |= (unsigned long long)bits << (4 * wi);
      }
      if (qn < 64) mm &= (1ull << qn) - 1ull;
      if (shading) mine += (uint32_t)__popcll(mm);
      while (mm) {
        const int j = __ffsll((long long)mm) - 1;
        mm &= mm - 1;
        Frag f;
        f.depth = q->depth[j];
        f.cover = q->cover[j];
        if (shading) {
          f.packed = q->packed[j];
          f.r = q->r[j];
          f.g = q->g[j];
          f.b = q->b[j];
          f.a = Pol::kViewZ ? __int_as_float(stage[q->tri[j]].xy2f.w) : q->vz[j];
          f.view_z = q->vz[j];
        }
        pol.fragment(p, pass, f, node0 + (uint32_t)j + 1u, tg);
      }
      if (shading) nfrag += (uint32_t)qn;
      qn = 0;
      qs = 0;
      __syncwarp();
    };

    // Coverage of one staged triangle against the warp's pixels (one lane per
    // pixel or sample); appends the covered fragments to the queue.
    auto cover_one = [&](int k) {
      const TriSetup& T = stage[k];
      const bool inb = lane_in_bbox(stage_bb[k], w);
      const int4 a = T.xy01, b = T.xy2f;
      const float4 zc = T.zc;
      uint32_t cover = 0;
      float zcen = 0.f;
      auto body = [&](auto etag) {
        using E = decltype(etag);
        const int bxp = w.px * 256, byp = w.py * 256;
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const int2 sp = SSN > 1 ? sample_pos<SSN>(w.sample) : sample_pos<S>(s);
          const EdgesT<E> e = edges_at<E>(a, b, bxp + sp.x, byp + sp.y);
          if (inside(e, b.z)) {
            const float z = depth_at(zc, e);
            if (__float_as_uint(z) < tg.depth[s]) cover |= 1u << s;
            if (S == 1) zcen = z;
          }
        }
        if (S > 1 && cover) zcen = depth_at(zc, edges_at<E>(a, b, bxp + 128, byp + 128));
      };
      if (inb) {
        if (b.z & kFlagSmall) body(int(0)); else body((long long)0);
      }
      const bool has = cover != 0;
      const uint32_t m = __ballot_sync(kFull, has);
      if (!m) return;
      const int cnt = __popc(m);
      if (qn + cnt > kQueue) flush();
      if (has) {
        const int j = qn + __popc(m & lt);
        q->tri[j] = (unsigned char)k;
        q->lane[j] = (unsigned char)w.lane;
        q->cover[j] = (unsigned char)cover;
        q->depth[j] = __float_as_uint(zcen);
      }
      qn += cnt;
    };

    // Coverage of a staged chunk by enumeration (no sample shading): the
    // pixels of every hit's bbox ∩ micro-tile are numbered hit by hit, row by
    // row, and lane g of each group of 32 tests pair g, reading the owner
    // lane's opaque depth by shuffle. Fragments enter the queue in lane order,
    // i.e. primitive order then pixel order, as the owners will consume them.
    auto cover_pairs = [&](int nh) {
      int n = 0, ox = 0, oy = 0, wd = 1;
      if (w.lane < nh) {
        const uint2 bb = stage_bb[w.lane];
        ox = max((int)(bb.x & 0xFFFF), w.rx0);
        oy = max((int)(bb.x >> 16), w.ry0);
        const int x1 = min(min((int)(bb.y & 0xFFFF), w.rx1), p.RW - 1);
        const int y1 = min(min((int)((bb.y >> 16) & 0x7FFF), w.ry1), p.RH - 1);
        wd = x1 - ox + 1;
        const int ht = y1 - oy + 1;
        n = (wd > 0 && ht > 0) ? wd * ht : 0;
      }
      int incl = n;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, o);
        if (w.lane >= o) incl += y;
      }
      const int total = __shfl_sync(kFull, incl, 31);
      if (w.lane < nh) {
        const int wdp = wd > 0 ? wd : 1;
        const int rx = n ? ox - w.rx0 : 0, ry = n ? oy - w.ry0 : 0;
        hr->packed[w.lane] = (uint32_t)(incl - n) | ((uint32_t)rx << 11) | ((uint32_t)ry << 14) |
                             ((uint32_t)wdp << 16) | ((uint32_t)((256 + wdp - 1) / wdp) << 20);
      }
      __syncwarp();
      for (int base = 0; base < total; base += 32) {
        const int g = base + w.lane;
        const bool act = g < total;
        // the hit holding pair g: the last hit whose prefix is <= g
        int lo = 0, hi = nh - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if ((int)(hr->packed[mid] & 0x7FFu) <= g) lo = mid; else hi = mid - 1;
        }
        const int k = lo;
        const uint32_t hk = hr->packed[k];
        const int r = g - (int)(hk & 0x7FFu);
        const int wdt = (int)((hk >> 16) & 0xFu);
        const int row = (r * (int)(hk >> 20)) >> 8;  // exact r / wdt for r < 32, wdt <= 8
        const int px = w.rx0 + (int)((hk >> 11) & 7u) + r - row * wdt, py = w.ry0 + (int)((hk >> 14) & 3u) + row;
        const int owner = act ? (py - w.ry0) * M::kW + (px - w.rx0) : 0;
        uint32_t od[S];
        if (p.has_opaque) {
#pragma unroll
          for (int s = 0; s < S; ++s) od[s] = __shfl_sync(kFull, tg.depth[s], owner);
        } else {
#pragma unroll
          for (int s = 0; s < S; ++s) od[s] = 0x3F800000u;  // no opaque pass: depth 1.0 everywhere
        }
        uint32_t cover = 0;
        float zcen = 0.f;
        if (act) {
          const TriSetup& T = stage[k];
          const int4 a = T.xy01, b = T.xy2f;
          const float4 zc = T.zc;
          const int bxp = px * 256, byp = py * 256;
          auto body = [&](auto etag) {
            using E = decltype(etag);
#pragma unroll
            for (int s = 0; s < S; ++s) {
              const int2 sp = sample_pos<S>(s);
              const EdgesT<E> e = edges_at<E>(a, b, bxp + sp.x, byp + sp.y);
              if (inside(e, b.z)) {
                const float z = depth_at(zc, e);
                if (__float_as_uint(z) < od[s]) cover |= 1u << s;
                if (S == 1) zcen = z;
              }
            }
            if (S > 1 && cover) zcen = depth_at(zc, edges_at<E>(a, b, bxp + 128, byp + 128));
          };
          if (b.z & kFlagSmall) body(int(0)); else body((long long)0);
        }
        const bool has = cover != 0;
        const uint32_t m = __ballot_sync(kFull, has);
        if (!m) continue;
        const int cnt = __popc(m);
        if (qn + cnt > kQueue) flush();
        if (has) {
          const int j = qn + __popc(m & lt);
          q->tri[j] = (unsigned char)k;
          q->lane[j] = (unsigned char)owner;
          q->cover[j] = (unsigned char)cover;
          q->depth[j] = __float_as_uint(zcen);
        }
        qn += cnt;
      }
      __syncwarp();
    };

    walk_pass<SSN == 1>(p, w, stage, stage_t, stage_bb, beg, end, [&](int nh) {
      if (SSN == 1) {
        cover_pairs(nh);
      } else {
        for (int k = 0; k < nh; ++k) cover_one(k);  // one lane per sample
      }
      // the next chunk replaces the staged records: shade now; WBOIT's
      // fragments also need their record's alpha, so it feeds every chunk
      if (Pol::kViewZ) flush(); else shade_pending();
    });
    flush();
  }

  pol.flush(p, w.valid);
  if (w.valid && p.color) {
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int s = 0; s < S; ++s) {
      c.x += tg.col[s].x;
      c.y += tg.col[s].y;
      c.z += tg.col[s].z;
      c.w += tg.col[s].w;
    }
    const float k = 1.0f / (float)S;
    store_color(p.color, p.color_half != 0, elem, make_float4(c.x * k, c.y * k, c.z * k, c.w * k));
  }
  if (w.lane == 0 && nfrag && p.frag_count) atomicAdd(p.frag_count, (unsigned long long)nfrag);
  if (SSN == 1 && p.lens) {
    const uint32_t mx = __reduce_max_sync(kFull, w.valid ? mine : 0u);
    // micro-tiles of edge tiles may lie wholly outside the image
    if (w.lane == 0 && w.rx0 < p.RW && w.ry0 < p.RH)
      p.lens[(size_t)(w.ry0 >> 2) * p.lens_stride + (w.rx0 >> 3)] = (uint8_t)min(mx, 255u);
  }
}

// The view of a multi-view launch that CTA `block` belongs to, and the CTA's
// index within that view's grid (block-uniform).
__device__ __forceinline__ int mv_view(const oit::MvRaster& mv, uint32_t block, int& cta) {
  int lo = 0, hi = mv.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (mv.cta_end[mid] > block) hi = mid; else lo = mid + 1;
  }
  cta = (int)(block - (lo ? mv.cta_end[lo - 1] : 0u));
  return lo;
}


// One view's pass: one CTA per kRasterWarpsPerBlock micro-tile warps, compiled
// for WPSM resident warps per SM with one coverage sample per lane (the
// register budget: 36 -> 56 registers, 32 -> 64).
template <template <int> class Policy, int S, int SSN, int WPSM = Policy<S>::kWarpsPerSM>
__global__ void __launch_bounds__(32 * kRasterWarpsPerBlock, (S == 1 ? WPSM : 24) / kRasterWarpsPerBlock)
    k_raster_transparent(RasterParams p) {
  raster_transparent_body<Policy, S, SSN>(p, (int)blockIdx.x);
}

// Several views' passes in one grid: the CTAs of view 0, then view 1, ...
// (the hardware hands out CTAs as earlier ones retire, so the views share the
// machine and small views fill what large ones leave).
template <template <int> class Policy, int S, int SSN>
__global__ void __launch_bounds__(32 * kRasterWarpsPerBlock,
                                  (S == 1 ? Policy<S>::kWarpsPerSM : 24) / kRasterWarpsPerBlock)
    k_raster_transparent_mv(const __grid_constant__ oit::MvRaster mv) {
  int cta;
  const int v = mv_view(mv, blockIdx.x, cta);
  raster_transparent_body<Policy, S, SSN>(mv.v[v], cta);
}

// ---------------------------------------------------------------------------
// Opaque pass: opaque.frag.glsl:30-35, depth LESS with write (main.cpp:542-547).
// ---------------------------------------------------------------------------
template <int S>
__device__ __forceinline__ void raster_opaque_body(const RasterParams& p, int cta) {
  __shared__ TriSetup stage_all[kRasterWarpsPerBlock * kStageSlots];
  __shared__ uint32_t stage_t_all[kRasterWarpsPerBlock * kStageSlots];
  __shared__ uint2 stage_bb_all[kRasterWarpsPerBlock * kStageSlots];
  const int warp = threadIdx.x >> 5;
  const WarpTile w = warp_tile<1>(p, cta);
  TriSetup* stage = stage_all + warp * kStageSlots;
  uint2* stage_bb = stage_bb_all + warp * kStageSlots;
  uint32_t dep[S];
  float4 col[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    dep[s] = w.valid ? p.depth[(size_t)s * p.P + w.pixel] : 0x3F800000u;
    col[s] = w.valid ? p.opaque_color[(size_t)s * p.P + w.pixel] : p.background;
  }
  const int tile = (int)((cta * kRasterWarpsPerBlock + warp) / oit::kWarpsPerTile) + p.tile_offset;
  walk_pass<true>(p, w, stage, stage_t_all + warp * kStageSlots, stage_bb, p.tile_begin[tile], p.tile_end[tile],
                  [&](int nh) {
    for (int k = 0; k < nh; ++k) {
      if (!lane_in_bbox(stage_bb[k], w)) continue;  // no warp-collective operation follows
      const TriSetup& T = stage[k];
      const int4 a = T.xy01, b = T.xy2f;
      const float4 zc = T.zc;
      auto body = [&](auto etag) {
        using E = decltype(etag);
        const int bxp = w.px * 256, byp = w.py * 256;
        uint32_t pass = 0;
        uint32_t zs[S];
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const int2 sp = sample_pos<S>(s);
          const EdgesT<E> e = edges_at<E>(a, b, bxp + sp.x, byp + sp.y);
          zs[s] = 0u;
          if (inside(e, b.z)) {
            const uint32_t z = __float_as_uint(depth_at(zc, e));
            zs[s] = z;
            if (z < dep[s]) pass |= 1u << s;
          }
        }
        if (!pass) return;
        const EdgesT<E> ec = edges_at<E>(a, b, bxp + 128, byp + 128);
        const Shade sh = shade(T, ec, nullptr);
        const float4 c = make_float4(sh.r, sh.g, sh.b, 1.0f);
#pragma unroll
        for (int s = 0; s < S; ++s)
          if (pass & (1u << s)) {
            dep[s] = zs[s];
            col[s] = c;
          }
      };
      if (b.z & kFlagSmall) body(int(0)); else body((long long)0);
    }
  });
  if (w.valid) {
#pragma unroll
    for (int s = 0; s < S; ++s) {
      p.depth[(size_t)s * p.P + w.pixel] = dep[s];
      p.opaque_color[(size_t)s * p.P + w.pixel] = col[s];
    }
  }
}

template <int S>
__global__ void __launch_bounds__(32 * kRasterWarpsPerBlock) k_raster_opaque(RasterParams p) {
  raster_opaque_body<S>(p, (int)blockIdx.x);
}

template <int S>
__global__ void __launch_bounds__(32 * kRasterWarpsPerBlock) k_raster_opaque_mv(const __grid_constant__ oit::MvRaster mv) {
  int cta;
  const int v = mv_view(mv, blockIdx.x, cta);
  raster_opaque_body<S>(mv.v[v], cta);
}

}  // namespace oitd

namespace oitd {

template <template <int> class Pol, int S, int SSN, int WPSM>
cudaError_t launch_transparent_w(const RasterParams& p, cudaStream_t s) {
  const size_t smem = (size_t)kRasterWarpsPerBlock *
                      (kWarpStageBytes + Pol<S>::smem_bytes_per_warp(p.L, p.coverage, p.record_fp32));
  if (smem > 48 * 1024) {
    // raise the kernel's dynamic shared memory cap once per device (never
    // while a CUDA graph is being captured after the first frame)
    static int cap_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || cap_set[dev] < (int)smem) {
      cudaError_t e = cudaFuncSetAttribute(k_raster_transparent<Pol, S, SSN, WPSM>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      if (dev >= 0 && dev < 64) cap_set[dev] = (int)smem;
    }
  }
  k_raster_transparent<Pol, S, SSN, WPSM><<<(unsigned)(p.tiles_x * p.tiles_y * SSN *
                                                       (oit::kWarpsPerTile / kRasterWarpsPerBlock)),
                                            32 * kRasterWarpsPerBlock, smem, s>>>(p);
  return cudaGetLastError();
}

// p.warps_per_sm 32 runs the 1x rasters whose default budget is 36 resident
// warps per SM at 32 (64 registers instead of 56); other values, the default.
template <template <int> class Pol, int S, int SSN>
cudaError_t launch_transparent_s(const RasterParams& p, cudaStream_t s) {
  constexpr int kDefault = Pol<S>::kWarpsPerSM;
  if constexpr (S == 1 && SSN == 1 && kDefault != 32) {
    if (p.warps_per_sm == 32) return launch_transparent_w<Pol, S, SSN, 32>(p, s);
  }
  return launch_transparent_w<Pol, S, SSN, kDefault>(p, s);
}

// Multi-view launch of one policy: mv.v[0..n) share S / SSN; the dynamic
// shared memory covers the largest per-warp policy state among them.
template <template <int> class Pol, int S, int SSN>
cudaError_t launch_transparent_mv_s(const oit::MvRaster& mv, cudaStream_t s) {
  size_t per_warp = 0;
  for (int i = 0; i < mv.n; ++i)
    per_warp = std::max(per_warp, Pol<S>::smem_bytes_per_warp(mv.v[i].L, mv.v[i].coverage, mv.v[i].record_fp32));
  const size_t smem = (size_t)kRasterWarpsPerBlock * (kWarpStageBytes + per_warp);
  if (smem > 48 * 1024) {
    static int cap_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || cap_set[dev] < (int)smem) {
      cudaError_t e = cudaFuncSetAttribute(k_raster_transparent_mv<Pol, S, SSN>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      if (dev >= 0 && dev < 64) cap_set[dev] = (int)smem;
    }
  }
  const uint32_t ctas = mv.n > 0 ? mv.cta_end[mv.n - 1] : 0u;
  if (!ctas) return cudaSuccess;
  k_raster_transparent_mv<Pol, S, SSN><<<ctas, 32 * kRasterWarpsPerBlock, smem, s>>>(mv);
  return cudaGetLastError();
}

template <template <int> class Pol>
cudaError_t launch_transparent_mv(const oit::MvRaster& mv, cudaStream_t s) {
  if (mv.n <= 0) return cudaSuccess;
  const RasterParams& p = mv.v[0];
  if (p.ssn > 1) {
    switch (p.ssn) {
      case 4: return launch_transparent_mv_s<Pol, 1, 4>(mv, s);
      case 8: return launch_transparent_mv_s<Pol, 1, 8>(mv, s);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (p.S) {
    case 1: return launch_transparent_mv_s<Pol, 1, 1>(mv, s);
    case 4: return launch_transparent_mv_s<Pol, 4, 1>(mv, s);
    case 8: return launch_transparent_mv_s<Pol, 8, 1>(mv, s);
    default: return cudaErrorInvalidValue;
  }
}

inline cudaError_t launch_opaque_mv(const oit::MvRaster& mv, cudaStream_t s) {
  if (mv.n <= 0) return cudaSuccess;
  const uint32_t ctas = mv.cta_end[mv.n - 1];
  if (!ctas) return cudaSuccess;
  constexpr int kThreads = 32 * kRasterWarpsPerBlock;
  switch (mv.v[0].S) {
    case 1: k_raster_opaque_mv<1><<<ctas, kThreads, 0, s>>>(mv); break;
    case 4: k_raster_opaque_mv<4><<<ctas, kThreads, 0, s>>>(mv); break;
    case 8: k_raster_opaque_mv<8><<<ctas, kThreads, 0, s>>>(mv); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <template <int> class Pol>
cudaError_t launch_transparent(const RasterParams& p, cudaStream_t s) {
  if (p.ssn > 1) {
    switch (p.ssn) {
      case 4: return launch_transparent_s<Pol, 1, 4>(p, s);
      case 8: return launch_transparent_s<Pol, 1, 8>(p, s);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (p.S) {
    case 1: return launch_transparent_s<Pol, 1, 1>(p, s);
    case 4: return launch_transparent_s<Pol, 4, 1>(p, s);
    case 8: return launch_transparent_s<Pol, 8, 1>(p, s);
    default: return cudaErrorInvalidValue;
  }
}

inline cudaError_t launch_opaque(const RasterParams& p, cudaStream_t s) {
  const unsigned grid = (unsigned)(p.tiles_x * p.tiles_y * (oit::kWarpsPerTile / kRasterWarpsPerBlock));
  constexpr int kThreads = 32 * kRasterWarpsPerBlock;
  switch (p.S) {
    case 1: k_raster_opaque<1><<<grid, kThreads, 0, s>>>(p); break;
    case 4: k_raster_opaque<4><<<grid, kThreads, 0, s>>>(p); break;
    case 8: k_raster_opaque<8><<<grid, kThreads, 0, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace oitd
