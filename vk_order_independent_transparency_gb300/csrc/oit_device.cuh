// Device-side building blocks shared by the engine's kernels: the triangle
// setup record, the fixed-point raster specification, Gooch shading and the
// exact sRGB8 quantisation. Every float operation on the raster/shading path
// uses an explicitly rounded intrinsic (__fmaf_rn, __fmul_rn, ...), which the
// compiler never contracts, so fragment depth and colour bits are identical
// on every run and equal to the CPU oracle's.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>
#include <cuda_runtime.h>

#include "oit_internal.h"
#include "srgb_tables.inc"

namespace oitd {

// Light direction normalize(vec3(-1, 2, 1)) of goochLighting
// (shaders/shaderCommon.glsl:36-44), rounded to float.
__device__ __forceinline__ float light_x() { return -0x1.a20bd8p-2f; }
__device__ __forceinline__ float light_y() { return 0x1.a20bd8p-1f; }
__device__ __forceinline__ float light_z() { return 0x1.a20bd8p-2f; }

// Sample positions in 1/256 pixel: centre for 1x, the standard Vulkan 4x and
// 8x patterns otherwise.
template <int S>
__device__ __forceinline__ int2 sample_pos(int s) {
  if (S == 1) return make_int2(128, 128);
  if (S == 4) {
    const int x[4] = {96, 224, 32, 160}, y[4] = {32, 96, 160, 224};
    return make_int2(x[s], y[s]);
  }
  const int x[8] = {144, 112, 208, 80, 48, 16, 176, 240};
  const int y[8] = {80, 176, 144, 48, 208, 112, 240, 16};
  return make_int2(x[s], y[s]);
}

// 96-byte triangle setup record, written by the setup kernel and staged into
// shared memory (cp.async) by the tile rasteriser.
struct __align__(16) TriSetup {
  int4 xy01;   // X0, Y0, X1, Y1 (1/256 px)
  int4 xy2f;   // X2, Y2, flags (bits 0-2 top-left per edge, bit 3 small, bits 8-15 alpha code), alpha (float bits)
  float4 zc;   // z0, z1 - z0, z2 - z0, 1 / area
  float4 n0;   // normal0 / w0 (xyz), red
  float4 n1;   // normal1 / w1 (xyz), green
  float4 n2;   // normal2 / w2 (xyz), blue
};
// Perspective terms used only for the view-space depth of WBOIT.
struct __align__(16) TriPersp {
  float4 q;    // 1/w0, 1/w1, 1/w2, 0
  float4 vzq;  // view z0 / w0, view z1 / w1, view z2 / w2, 0
};
constexpr int kFlagSmall = 8;     // bbox extent < 64 px: edge functions fit in int32
constexpr int kSmallExtent = 1 << 14;

// Edge values at a sample (px, py) in 1/256 pixel units. Edge i is opposite
// vertex i and runs from vertex (i+1)%3 to (i+2)%3. For triangles whose bbox
// spans less than 2^14 units every product stays below 2^28, so the int32
// path computes exactly the same values as the int64 one.
template <typename E>
struct EdgesT {
  E e0, e1, e2;
};
using Edges = EdgesT<long long>;

template <typename E>
__device__ __forceinline__ EdgesT<E> edges_at(const int4& a, const int4& b, int px, int py) {
  EdgesT<E> r;
  const int X0 = a.x, Y0 = a.y, X1 = a.z, Y1 = a.w, X2 = b.x, Y2 = b.y;
  r.e0 = (E)(X2 - X1) * (E)(py - Y1) - (E)(Y2 - Y1) * (E)(px - X1);
  r.e1 = (E)(X0 - X2) * (E)(py - Y2) - (E)(Y0 - Y2) * (E)(px - X2);
  r.e2 = (E)(X1 - X0) * (E)(py - Y0) - (E)(Y1 - Y0) * (E)(px - X0);
  return r;
}

__device__ __forceinline__ Edges edges_at(const int4& a, const int4& b, int px, int py) {
  return edges_at<long long>(a, b, px, py);
}

template <typename E>
__device__ __forceinline__ bool inside(const EdgesT<E>& e, int tl) {
  return (e.e0 > 0 || (e.e0 == 0 && (tl & 1))) && (e.e1 > 0 || (e.e1 == 0 && (tl & 2))) &&
         (e.e2 > 0 || (e.e2 == 0 && (tl & 4)));
}

__device__ __forceinline__ float to_float(long long v) { return __ll2float_rn(v); }
__device__ __forceinline__ float to_float(int v) { return __int2float_rn(v); }

// Window depth at the edge values (screen-linear interpolation), clamped to [0,1].
template <typename E>
__device__ __forceinline__ float depth_at(const float4& zc, const EdgesT<E>& e) {
  const float b1 = __fmul_rn(to_float(e.e1), zc.w);
  const float b2 = __fmul_rn(to_float(e.e2), zc.w);
  float z = __fmaf_rn(b2, zc.z, __fmaf_rn(b1, zc.y, zc.x));
  z = (z > 0.0f) ? z : 0.0f;
  z = (z < 1.0f) ? z : 1.0f;
  return z;
}

// Exact sRGB8 quantisation tables (gen_srgb_tables.py).
struct SrgbTables {
  float thr[256];
  unsigned char bucket[4096];
  float dec[256];
};
// One copy per translation unit (no relocatable device code needed).
static __device__ SrgbTables g_srgb = {OIT_SRGB_THR_INIT, OIT_SRGB_BUCKET_INIT, OIT_SRGB_DEC_INIT};

__device__ __forceinline__ uint32_t srgb_encode(float c) {
  if (!(c > 0.0f)) return 0u;
  if (c >= 1.0f) return 255u;
  int idx = (int)__fmul_rn(c, 4096.0f);
  idx = idx < 4095 ? idx : 4095;
  uint32_t code = __ldg(&g_srgb.bucket[idx]);
  code += (c >= __ldg(&g_srgb.thr[code])) ? 1u : 0u;
  return code;
}

__device__ __forceinline__ float srgb_decode(uint32_t code) { return __ldg(&g_srgb.dec[code & 255u]); }

// Perspective-correct Gooch shading (shaders/shaderCommon.glsl:36-56) at the
// edge values e; returns linear unpremultiplied rgb, and the interpolated view
// space z when P is given.
struct Shade {
  float r, g, b, view_z;
};

template <typename E>
__device__ __forceinline__ Shade shade(const TriSetup& T, const EdgesT<E>& e, const TriPersp* P) {
  const float inv_area = T.zc.w;
  const float b0 = __fmul_rn(to_float(e.e0), inv_area);
  const float b1 = __fmul_rn(to_float(e.e1), inv_area);
  const float b2 = __fmul_rn(to_float(e.e2), inv_area);
  const float4 n0 = T.n0, n1 = T.n1, n2 = T.n2;
  const float nx = __fmaf_rn(b2, n2.x, __fmaf_rn(b1, n1.x, __fmul_rn(b0, n0.x)));
  const float ny = __fmaf_rn(b2, n2.y, __fmaf_rn(b1, n1.y, __fmul_rn(b0, n0.y)));
  const float nz = __fmaf_rn(b2, n2.z, __fmaf_rn(b1, n1.z, __fmul_rn(b0, n0.z)));
  const float len2 = __fmaf_rn(nz, nz, __fmaf_rn(ny, ny, __fmul_rn(nx, nx)));
  const float d = __fmaf_rn(nz, light_z(), __fmaf_rn(ny, light_y(), __fmul_rn(nx, light_x())));
  const float c = (len2 > 0.0f) ? __fdiv_rn(d, __fsqrt_rn(len2)) : 0.0f;
  const float warmth = __fmaf_rn(c, 0.5f, 0.5f);
  Shade s;
  s.r = __fmul_rn(n0.w, warmth);
  s.g = __fmul_rn(n1.w, __fmaf_rn(0.75f, warmth, 0.25f));
  s.b = __fmul_rn(n2.w, __fmaf_rn(0.25f, warmth, 0.75f));
  s.view_z = 0.0f;
  if (P) {
    const float4 q = P->q, vz = P->vzq;
    const float num = __fmaf_rn(b2, vz.z, __fmaf_rn(b1, vz.y, __fmul_rn(b0, vz.x)));
    const float den = __fmaf_rn(b2, q.z, __fmaf_rn(b1, q.y, __fmul_rn(b0, q.x)));
    s.view_z = __fdiv_rn(num, den);
  }
  return s;
}

__device__ __forceinline__ uint32_t pack_rgba8(const Shade& s, uint32_t alpha_code) {
  return srgb_encode(s.r) | (srgb_encode(s.g) << 8) | (srgb_encode(s.b) << 16) | (alpha_code << 24);
}

// Premultiplied "over" helpers in FP32 (shaderCommon.glsl:108-124, blend state main.cpp:548-558).
__device__ __forceinline__ float4 decode_premult(uint32_t packed) {
  const float a = (float)(packed >> 24) * (1.0f / 255.0f);
  return make_float4(srgb_decode(packed) * a, srgb_decode(packed >> 8) * a, srgb_decode(packed >> 16) * a, a);
}

// color = color over base (doBlend)
__device__ __forceinline__ void blend_under(float4& color, const float4& base) {
  const float k = 1.0f - color.w;
  color.x = fmaf(k, base.x, color.x);
  color.y = fmaf(k, base.y, color.y);
  color.z = fmaf(k, base.z, color.z);
  color.w = fmaf(k, base.w, color.w);
}

// dst = src over dst (hardware ONE, ONE_MINUS_SRC_ALPHA)
__device__ __forceinline__ void rop_over(float4& dst, const float4& src) {
  const float k = 1.0f - src.w;
  dst.x = fmaf(k, dst.x, src.x);
  dst.y = fmaf(k, dst.y, src.y);
  dst.z = fmaf(k, dst.z, src.z);
  dst.w = fmaf(k, dst.w, src.w);
}

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t bits) { atomicOr(err, bits); }

// Colour target element: float4, or (OIT_FLAG_HALF_COLOR) four halves.
__device__ __forceinline__ void store_color(float4* base, bool half, size_t i, float4 c) {
  if (half) {
    const __half2 lo = __floats2half2_rn(c.x, c.y), hi = __floats2half2_rn(c.z, c.w);
    reinterpret_cast<uint2*>(base)[i] =
        make_uint2(*reinterpret_cast<const uint32_t*>(&lo), *reinterpret_cast<const uint32_t*>(&hi));
  } else {
    base[i] = c;
  }
}

// Read once by the composite: streaming loads.
__device__ __forceinline__ float4 load_color(const float4* base, bool half, size_t i) {
  if (half) {
    const uint2 v = __ldcs(reinterpret_cast<const uint2*>(base) + i);
    const float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
    const float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
    return make_float4(lo.x, lo.y, hi.x, hi.y);
  }
  return __ldcs(base + i);
}

// Resolved premultiplied colour to the RGBA8 sRGB output (alpha stays
// linear), plus the optional linear copy.
__device__ __forceinline__ void write_rgba8(uint8_t* out8, float4* out_linear, uint32_t o, float4 c) {
  const float a = fminf(fmaxf(c.w, 0.0f), 1.0f);
  const uint32_t ac = (uint32_t)__float2int_rn(a * 255.0f);
  const uint32_t v = srgb_encode(c.x) | (srgb_encode(c.y) << 8) | (srgb_encode(c.z) << 16) | (ac << 24);
  reinterpret_cast<uint32_t*>(out8)[o] = v;
  if (out_linear) out_linear[o] = c;
}

}  // namespace oitd
