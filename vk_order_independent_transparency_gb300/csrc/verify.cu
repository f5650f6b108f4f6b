// FP64 verification resolve.
//
// The COMPOSITE pass of a frame recomputed in double precision from the
// frame's own A-buffer, aux words and tail-blended colour target: the same
// gathers and sorts as composite.cu (the reference's bubbleSort with its
// swap-on-equal, insertionSort / insertionSortTail, coverage resolve,
// oitCompositeDefines.glsl:51-139, oitSimple.frag.glsl:142-159), with
// doBlend / doBlendPacked (shaderCommon.glsl:108-124) and the blend onto the
// colour target (ONE, ONE_MINUS_SRC_ALPHA, main.cpp:548-558) evaluated in
// FP64, then the MSAA / supersample box resolve. It checks the FP32 (and
// FP16 colour target) production resolve; it is never part of a frame. Depth
// keys and sort order stay exact integers, as in the production kernels.
//
// The sRGB decode table is computed on the host in double, with the
// formula of unPremultSRGBToLinear (shaderCommon.glsl:83-93), and passed in
// the parameters, so the kernel blends the same decoded values as a CPU
// restatement in double.
#include <cmath>
#include <cuda_fp16.h>

#include "oit_device.cuh"
#include "oit_internal.h"

namespace oit {

namespace {

constexpr int kMaxL = 32;
constexpr uint32_t kEmptyWord = 0xFFFFFFFFu;

struct D4 {
  double r, g, b, a;
};

struct VerifyTables {
  double dec[256];  // sRGB8 code -> linear
  float thr[256];   // thr[k]: smallest linear value encoding to k + 1 (k < 255)
};

struct VerifyParams {
  CompositeParams c;
  VerifyTables t;
  double* out_linear;  // [W*H] double4 premultiplied linear
};

__device__ __forceinline__ D4 zero4() { return D4{0.0, 0.0, 0.0, 0.0}; }

__device__ __forceinline__ D4 premult_packed(const VerifyTables& t, uint32_t packed) {
  const double a = (double)(packed >> 24) / 255.0;
  return D4{t.dec[packed & 255u] * a, t.dec[(packed >> 8) & 255u] * a, t.dec[(packed >> 16) & 255u] * a, a};
}

__device__ __forceinline__ D4 premult_float4(const float* c) {
  const double a = (double)c[3];
  return D4{(double)c[0] * a, (double)c[1] * a, (double)c[2] * a, a};
}

// doBlend: color = color over base, separate multiply and add
__device__ __forceinline__ void blend_under(D4& color, const D4& base) {
  const double k = __dsub_rn(1.0, color.a);
  color.r = __dadd_rn(color.r, __dmul_rn(k, base.r));
  color.g = __dadd_rn(color.g, __dmul_rn(k, base.g));
  color.b = __dadd_rn(color.b, __dmul_rn(k, base.b));
  color.a = __dadd_rn(color.a, __dmul_rn(k, base.a));
}

// dst = src + (1 - src.a) dst
__device__ __forceinline__ void rop_over(D4& dst, const D4& src) {
  const double k = __dsub_rn(1.0, src.a);
  dst.r = __dadd_rn(src.r, __dmul_rn(k, dst.r));
  dst.g = __dadd_rn(src.g, __dmul_rn(k, dst.g));
  dst.b = __dadd_rn(src.b, __dmul_rn(k, dst.b));
  dst.a = __dadd_rn(src.a, __dmul_rn(k, dst.a));
}

__device__ __forceinline__ bool dge(uint32_t a, uint32_t b) { return __uint_as_float(a) >= __uint_as_float(b); }
__device__ __forceinline__ bool dlt(uint32_t a, uint32_t b) { return __uint_as_float(a) < __uint_as_float(b); }

// Sort entries: colour word (packed RGBA8, or an index naming a float colour),
// depth bits, coverage mask.
struct Entries {
  uint32_t c[kMaxL], d[kMaxL], m[kMaxL];
};

// bubbleSort, oitCompositeDefines.glsl:51-89 (swap on >=)
__device__ void bubble_sort(Entries& a, int n) {
  for (int i = n - 2; i >= 0; --i)
    for (int j = 0; j <= i; ++j)
      if (dge(a.d[j], a.d[j + 1])) {
        uint32_t t;
        t = a.c[j]; a.c[j] = a.c[j + 1]; a.c[j + 1] = t;
        t = a.d[j]; a.d[j] = a.d[j + 1]; a.d[j + 1] = t;
        t = a.m[j]; a.m[j] = a.m[j + 1]; a.m[j + 1] = t;
      }
}

// insertionSortTail, oitCompositeDefines.glsl:94-139, on a full array of L
// entries: returns the colour word of the entry that leaves the array (the
// item itself when it is not nearer than the last entry).
__device__ uint32_t insertion_sort_tail(Entries& a, int L, uint32_t ic, uint32_t id, uint32_t im) {
  if (!dlt(id, a.d[L - 1])) return ic;
  const uint32_t last = a.c[L - 1];
  int pos = L - 1;
  while (pos > 0 && dlt(id, a.d[pos - 1])) {
    a.c[pos] = a.c[pos - 1];
    a.d[pos] = a.d[pos - 1];
    a.m[pos] = a.m[pos - 1];
    --pos;
  }
  a.c[pos] = ic;
  a.d[pos] = id;
  a.m[pos] = im;
  return last;
}

struct Colour {
  const VerifyTables* t;
  const uint4* pool;  // RGBA32F linked-list nodes (colour word = node index), else null
  __device__ D4 operator()(uint32_t c) const {
    if (pool) {
      const uint4 v = pool[2 * (size_t)c];
      const float f[4] = {__uint_as_float(v.x), __uint_as_float(v.y), __uint_as_float(v.z), __uint_as_float(v.w)};
      return premult_float4(f);
    }
    return premult_packed(*t, c);
  }
};

__device__ D4 blend_entries(const Entries& a, int n, int coverage, int S, const Colour& col) {
  D4 sum = zero4();
  if (!coverage) {
    for (int i = 0; i < n; ++i) blend_under(sum, col(a.c[i]));
    return sum;
  }
  for (int s = 0; s < S; ++s) {
    D4 sc = zero4();
    for (int i = 0; i < n; ++i)
      if ((a.m[i] >> s) & 1u) blend_under(sc, col(a.c[i]));
    sum.r += sc.r;
    sum.g += sc.g;
    sum.b += sc.b;
    sum.a += sc.a;
  }
  return D4{sum.r / S, sum.g / S, sum.b / S, sum.a / S};
}

// One A-buffer element (pixel, or sample with sample shading).
__device__ D4 composite_element(const VerifyParams& vp, Alg alg, uint32_t eaux, size_t abase, size_t abase_loop) {
  const CompositeParams& p = vp.c;
  const int L = p.L;
  Entries a;
  switch (alg) {
    case Alg::Simple:
    case Alg::Spinlock:
    case Alg::Interlock: {
      // oitSimple.frag.glsl:115-169 (Spinlock, Interlock: the same composite)
      int n = (int)min(p.aux[eaux], (uint32_t)L);
      for (int i = 0; i < n; ++i) {
        const size_t o = abase + (size_t)i * p.P;
        if (p.coverage) {
          const uint4 r = reinterpret_cast<const uint4*>(p.abuf)[o];
          a.c[i] = r.x; a.d[i] = r.y; a.m[i] = r.z;
        } else {
          const uint2 r = reinterpret_cast<const uint2*>(p.abuf)[o];
          a.c[i] = r.x; a.d[i] = r.y; a.m[i] = 0;
        }
      }
      bubble_sort(a, n);
      return blend_entries(a, n, p.coverage, p.S, Colour{&vp.t, nullptr});
    }
    case Alg::LinkedList: {
      // oitLinkedList.frag.glsl:106-172
      const uint4* pool = reinterpret_cast<const uint4*>(p.abuf);
      const bool f32 = p.record_fp32 != 0;
      const Colour col{&vp.t, f32 ? pool : nullptr};
      auto node = [&](uint32_t off, uint32_t& c, uint32_t& d, uint32_t& m) {
        if (f32) {
          const uint4 nd = pool[2 * (size_t)off + 1];
          c = off; d = nd.x; m = nd.y;
          return nd.z;
        }
        const uint4 nd = pool[off];
        c = nd.x; d = nd.y; m = nd.z;
        return nd.w;
      };
      uint32_t off = p.aux[eaux];
      if (off >= p.capacity) off = 0;
      int n = 0;
      uint32_t guard = p.capacity;  // lists built this frame are acyclic
      while (off != 0 && n < L && guard-- != 0) {
        const uint32_t next = node(off, a.c[n], a.d[n], a.m[n]);
        ++n;
        off = next < p.capacity ? next : 0u;
      }
      bubble_sort(a, n);
      D4 tail = zero4();
      while (off != 0 && guard-- != 0) {
        uint32_t ic, id, im;
        const uint32_t next = node(off, ic, id, im);
        const uint32_t ev = insertion_sort_tail(a, L, ic, id, im);
        if (p.tail) blend_under(tail, col(ev));  // the tail ignores coverage (:137-138)
        off = next < p.capacity ? next : 0u;
      }
      D4 sum = blend_entries(a, n, p.coverage, p.S, col);
      blend_under(sum, tail);
      return sum;
    }
    case Alg::Loop: {
      // oitLoop.frag.glsl:191-222
      int n = 0;
      while (n < L && p.abuf[abase_loop + (size_t)n * p.P] != kEmptyWord) ++n;
      D4 sum = zero4();
      for (int i = 0; i < n; ++i) blend_under(sum, premult_packed(vp.t, p.abuf[abase_loop + (size_t)(L + i) * p.P]));
      return sum;
    }
    case Alg::Loop64: {
      // oitLoop64.frag.glsl:162-183; RGBA32F: a float4 payload block after the keys
      const uint2* ab = reinterpret_cast<const uint2*>(p.abuf);
      const float4* pay = p.record_fp32 ? reinterpret_cast<const float4*>(ab + (size_t)p.ssn * L * p.P) : nullptr;
      D4 sum = zero4();
      for (int i = 0; i < L; ++i) {
        const uint2 k = ab[abase + (size_t)i * p.P];
        if (k.y == kEmptyWord) break;
        if (pay) {
          const float4 c = pay[abase + (size_t)i * p.P];
          const float f[4] = {c.x, c.y, c.z, c.w};
          blend_under(sum, premult_float4(f));
        } else {
          blend_under(sum, premult_packed(vp.t, k.x));
        }
      }
      return sum;
    }
    default: return zero4();
  }
}

__device__ D4 load_target(const CompositeParams& p, size_t i) {
  if (p.color_half) {
    const uint2 v = reinterpret_cast<const uint2*>(p.color)[i];
    const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
    const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
    return D4{lo.x, lo.y, hi.x, hi.y};
  }
  const float4 c = p.color[i];
  return D4{c.x, c.y, c.z, c.w};
}

// WBOIT composite, oitWeighted.frag.glsl:98-108 with blend ONE_MINUS_SRC_ALPHA /
// SRC_ALPHA (main.cpp:578-588), from the stored accumulators.
__device__ D4 weighted_sample(const CompositeParams& p, size_t o) {
  D4 a;
  double rv;
  if (p.weighted_fp32) {
    const float4 v = reinterpret_cast<const float4*>(p.accum)[o];
    a = D4{v.x, v.y, v.z, v.w};
    rv = reinterpret_cast<const float*>(p.reveal)[o];
  } else {
    const uint2 v = reinterpret_cast<const uint2*>(p.accum)[o];
    const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
    const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
    a = D4{lo.x, lo.y, hi.x, hi.y};
    rv = __half2float(reinterpret_cast<const __half*>(p.reveal)[o]);
  }
  D4 base;
  if (p.has_opaque) {
    const float4 c = p.opaque_color[o];
    base = D4{c.x, c.y, c.z, c.w};
  } else {
    base = D4{p.background.x, p.background.y, p.background.z, p.background.w};
  }
  const double d = a.a > 1e-5 ? a.a : 1e-5;
  const double ia = 1.0 - rv;
  return D4{(a.r / d) * ia + base.r * rv, (a.g / d) * ia + base.g * rv, (a.b / d) * ia + base.b * rv,
            rv * ia + base.a * rv};
}

__device__ uint32_t encode_code(const VerifyTables& t, double c) {
  int lo = 0, hi = 255;  // number of thresholds <= c
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (c >= (double)t.thr[mid]) lo = mid + 1; else hi = mid;
  }
  return (uint32_t)lo;
}

__global__ void __launch_bounds__(128) k_composite_fp64(VerifyParams vp, Alg alg) {
  const CompositeParams& p = vp.c;
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 4 + (threadIdx.x >> 5);
  if (x >= p.W || y >= p.H) return;
  D4 acc = zero4();
  int count = 0;
  for (int dy = 0; dy < p.ss; ++dy)
    for (int dx = 0; dx < p.ss; ++dx) {
      const uint32_t pixel = (uint32_t)(y * p.ss + dy) * (uint32_t)p.RW + (uint32_t)(x * p.ss + dx);
      if (alg == Alg::Weighted) {
        for (int s = 0; s < p.S; ++s, ++count) {
          const D4 c = weighted_sample(p, (size_t)s * p.P + pixel);
          acc.r += c.r; acc.g += c.g; acc.b += c.b; acc.a += c.a;
        }
        continue;
      }
      for (int s = 0; s < p.ssn; ++s, ++count) {
        const uint32_t eaux = (uint32_t)s * p.P + pixel;
        const size_t abase = (size_t)s * p.L * p.P + pixel;
        const size_t abase_loop = (size_t)s * 2 * p.L * p.P + pixel;
        const D4 sum = composite_element(vp, alg, eaux, abase, abase_loop);
        D4 c = load_target(p, eaux);
        rop_over(c, sum);
        acc.r += c.r; acc.g += c.g; acc.b += c.b; acc.a += c.a;
      }
    }
  const double k = 1.0 / (double)count;
  acc = D4{acc.r * k, acc.g * k, acc.b * k, acc.a * k};
  const size_t o = (size_t)y * p.W + x;
  if (vp.out_linear) {
    double* ol = vp.out_linear + 4 * o;
    ol[0] = acc.r;
    ol[1] = acc.g;
    ol[2] = acc.b;
    ol[3] = acc.a;
  }
  if (p.out_rgba8) {
    double al = acc.a > 0.0 ? acc.a : 0.0;
    al = al < 1.0 ? al : 1.0;
    const uint32_t ac = (uint32_t)__double2int_rn(al * 255.0);
    reinterpret_cast<uint32_t*>(p.out_rgba8)[o] =
        encode_code(vp.t, acc.r) | (encode_code(vp.t, acc.g) << 8) | (encode_code(vp.t, acc.b) << 16) | (ac << 24);
  }
}

const VerifyTables& host_tables() {
  static const VerifyTables t = [] {
    VerifyTables v{};
    float dec32[256];
    srgb_host_tables(v.thr, dec32);
    for (int c = 0; c < 256; ++c) {
      // unPremultSRGBToLinear (shaderCommon.glsl:83-93) in double
      const double s = (double)c / 255.0;
      v.dec[c] = (s < 0.04045) ? s / 12.92 : std::pow((s + 0.055) / 1.055, 2.4);
    }
    return v;
  }();
  return t;
}

}  // namespace

cudaError_t launch_composite_fp64(Alg alg, const CompositeParams& c, double* out_linear, cudaStream_t s) {
  if (c.L > kMaxL) return cudaErrorInvalidValue;
  VerifyParams vp;
  vp.c = c;
  vp.t = host_tables();
  vp.out_linear = out_linear;
  const dim3 grid((c.W + 31) / 32, (c.H + 3) / 4);
  k_composite_fp64<<<grid, 128, 0, s>>>(vp, alg);
  return cudaGetLastError();
}

}  // namespace oit
