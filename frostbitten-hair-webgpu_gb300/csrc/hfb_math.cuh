// Device-side WGSL built-ins with a fixed fp32 evaluation order.
//
// The library is compiled with -fmad=false, -prec-div=true and
// -prec-sqrt=true, so every expression below is one IEEE operation at a time
// with no fused multiply-add.  The conventions are those of WGSL as the hair
// passes use it (src/passes/_shaderSnippets/shaderSnippets.wgls.ts:61-166):
//   dot(a,b) = ((a.x*b.x + a.y*b.y) + a.z*b.z); length = sqrt(dot(v,v));
//   normalize(v) = v / length(v); mix(a,b,t) = a*(1-t) + b*t;
//   fract(x) = x - floor(x); min/max = fminf/fmaxf;
//   mat4 * vec4 (column-major) = ((c0*v.x + c1*v.y) + c2*v.z) + c3*v.w;
//   u32(f32) / i32(f32) saturate, truncate toward zero, NaN -> 0.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace hfb {

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

__device__ __forceinline__ f2 mk2(float x, float y) { return {x, y}; }
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f4 mk4(float x, float y, float z, float w) { return {x, y, z, w}; }
__device__ __forceinline__ f4 ld4(const float4 v) { return {v.x, v.y, v.z, v.w}; }
__device__ __forceinline__ f3 xyz(f4 a) { return {a.x, a.y, a.z}; }

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float sat(float x) { return clampf(x, 0.0f, 1.0f); }
__device__ __forceinline__ float mixf(float a, float b, float t) {
  return fadd(fmul(a, fsub(1.0f, t)), fmul(b, t));
}
__device__ __forceinline__ float fractf(float x) { return fsub(x, floorf(x)); }
__device__ __forceinline__ uint32_t clampu(uint32_t x, uint32_t lo, uint32_t hi) {
  return min(max(x, lo), hi);
}
__device__ __forceinline__ uint32_t f2u(float f) { return __float2uint_rz(f); }
__device__ __forceinline__ int32_t f2i(float f) { return __float2int_rz(f); }

__device__ __forceinline__ f2 add2(f2 a, f2 b) { return {fadd(a.x, b.x), fadd(a.y, b.y)}; }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { return {fsub(a.x, b.x), fsub(a.y, b.y)}; }
__device__ __forceinline__ f2 mul2s(f2 a, float s) { return {fmul(a.x, s), fmul(a.y, s)}; }
__device__ __forceinline__ f2 div2s(f2 a, float s) { return {a.x / s, a.y / s}; }
__device__ __forceinline__ float dot2(f2 a, f2 b) { return fadd(fmul(a.x, b.x), fmul(a.y, b.y)); }
__device__ __forceinline__ float len2(f2 a) { return sqrtf(dot2(a, a)); }
__device__ __forceinline__ f2 norm2(f2 a) { float l = len2(a); return {a.x / l, a.y / l}; }

__device__ __forceinline__ f3 add3(f3 a, f3 b) { return {fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return {fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)}; }
__device__ __forceinline__ f3 mul3(f3 a, f3 b) { return {fmul(a.x, b.x), fmul(a.y, b.y), fmul(a.z, b.z)}; }
__device__ __forceinline__ f3 mul3s(f3 a, float s) { return {fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)}; }
__device__ __forceinline__ f3 div3(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ f3 div3s(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) {
  return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z));
}
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ f3 norm3(f3 a) { float l = len3(a); return {a.x / l, a.y / l, a.z / l}; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return {fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
          fsub(fmul(a.x, b.y), fmul(a.y, b.x))};
}
__device__ __forceinline__ f3 mix3(f3 a, f3 b, float t) {
  return {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)};
}
__device__ __forceinline__ f3 sat3(f3 a) { return {sat(a.x), sat(a.y), sat(a.z)}; }
__device__ __forceinline__ f4 mix4(f4 a, f4 b, float t) {
  return {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t), mixf(a.w, b.w, t)};
}

// mat4 (column-major, 16 floats) * vec4
__device__ __forceinline__ f4 m4v(const float* m, f4 v) {
  f4 r;
  r.x = fadd(fadd(fadd(fmul(m[0], v.x), fmul(m[4], v.y)), fmul(m[8], v.z)), fmul(m[12], v.w));
  r.y = fadd(fadd(fadd(fmul(m[1], v.x), fmul(m[5], v.y)), fmul(m[9], v.z)), fmul(m[13], v.w));
  r.z = fadd(fadd(fadd(fmul(m[2], v.x), fmul(m[6], v.y)), fmul(m[10], v.z)), fmul(m[14], v.w));
  r.w = fadd(fadd(fadd(fmul(m[3], v.x), fmul(m[7], v.y)), fmul(m[11], v.z)), fmul(m[15], v.w));
  return r;
}

// projectVertex, shaderSnippets.wgls.ts:92-96
__device__ __forceinline__ f3 projectVertex(const float* mvp, f4 pos) {
  f4 c = m4v(mvp, pos);
  return {c.x / c.w, c.y / c.w, c.z / c.w};
}

// projectPointToLine, shaderSnippets.wgls.ts:99-105
__device__ __forceinline__ f2 projectPointToLine(f2 l1, f2 l2, f2 p) {
  f2 ab = sub2(l2, l1);
  f2 ac = sub2(p, l1);
  float d1 = dot2(ab, ac);
  float d2 = dot2(ab, ab);
  return add2(l1, div2s(mul2s(ab, d1), d2));
}

// ndc2viewportPx, shaderSnippets.wgls.ts:107-110
__device__ __forceinline__ f2 ndc2viewportPx(f2 size, f3 pos) {
  f2 p01 = {fadd(fmul(pos.x, 0.5f), 0.5f), fadd(fmul(pos.y, 0.5f), 0.5f)};
  return {fmul(p01.x, size.x), fmul(p01.y, size.y)};
}

// remapToIndices, shaderSnippets.wgls.ts:124-130
__device__ __forceinline__ float remapToIndices(uint32_t maxIdx, float t, uint32_t& i0, uint32_t& i1) {
  float a = fmul(t, fsub((float)maxIdx, 1.0f));
  uint32_t au = f2u(a);
  i0 = clampu(au, 0u, maxIdx - 1u);
  i1 = clampu(au + 1u, 0u, maxIdx - 1u);
  return fractf(a);
}

// getDepthBin, shaderSnippets.wgls.ts:152-160
__device__ __forceinline__ uint32_t getDepthBin(uint32_t binCount, float d0, float d1, float pixelDepth) {
  float span = fabsf(fsub(d1, d0));
  float t = fsub(pixelDepth, d0) / span;
  return clampu(f2u(fmul(t, (float)binCount)), 0u, binCount - 1u);
}

// edgeFunction, swRasterizeHair.wgsl.ts:128-130
__device__ __forceinline__ float edgeFunction(f2 v0, f2 v1, f2 p) {
  return fsub(fmul(fsub(p.x, v0.x), fsub(v1.y, v0.y)), fmul(fsub(p.y, v0.y), fsub(v1.x, v0.x)));
}

// ProjectedHairSegment, swRasterizeHair.wgsl.ts:27-33
struct ProjSeg {
  f2 v00, v01, v10, v11;
  f4 depthsProj;
};

// interpolateHairQuad, swRasterizeHair.wgsl.ts:170-196
__device__ __forceinline__ f2 interpolateHairQuad(const ProjSeg& s, f2 c) {
  f2 sm = div2s(add2(s.v00, s.v01), 2.0f);
  f2 em = div2s(add2(s.v10, s.v11), 2.0f);
  f2 cp = projectPointToLine(sm, em, c);
  float d1 = len2(sub2(cp, sm)) / len2(sub2(sm, em));
  float widthStart = len2(sub2(s.v00, s.v01));
  float widthEnd = fmul(widthStart, dot2(norm2(sub2(s.v00, s.v01)), norm2(sub2(s.v10, s.v11))));
  float expectedWidth = mixf(widthStart, widthEnd, d1);
  f2 e1 = projectPointToLine(s.v00, s.v10, c);
  float d0 = len2(sub2(c, e1)) / expectedWidth;
  return {sat(d0), sat(d1)};
}

// The pixel-independent parts of interpolateHairQuad, computed once per
// segment with exactly the operations interpolateHairQuad performs, so the
// per-pixel remainder (interpolateHairQuadPre) returns identical values.
struct QuadConst {
  f2 sm, ab;          // start-edge midpoint; end midpoint - start midpoint
  float d2, lse;      // dot(ab, ab); length(sm - em)
  float wS, wE;       // widthStart, widthEnd
  f2 ab2;             // v10 - v00
  float d22, pad;     // dot(ab2, ab2)
};

__device__ __forceinline__ QuadConst quadConst(const ProjSeg& s) {
  QuadConst q;
  q.sm = div2s(add2(s.v00, s.v01), 2.0f);
  f2 em = div2s(add2(s.v10, s.v11), 2.0f);
  q.ab = sub2(em, q.sm);
  q.d2 = dot2(q.ab, q.ab);
  q.lse = len2(sub2(q.sm, em));
  q.wS = len2(sub2(s.v00, s.v01));
  q.wE = fmul(q.wS, dot2(norm2(sub2(s.v00, s.v01)), norm2(sub2(s.v10, s.v11))));
  q.ab2 = sub2(s.v10, s.v00);
  q.d22 = dot2(q.ab2, q.ab2);
  q.pad = 0.0f;
  return q;
}

// interpolateHairQuad with the per-segment constants precomputed
__device__ __forceinline__ f2 interpolateHairQuadPre(const QuadConst& q, f2 v00, f2 c) {
  // cp = projectPointToLine(sm, em, c)
  f2 ac = sub2(c, q.sm);
  f2 cp = add2(q.sm, div2s(mul2s(q.ab, dot2(q.ab, ac)), q.d2));
  float d1 = len2(sub2(cp, q.sm)) / q.lse;
  float expectedWidth = mixf(q.wS, q.wE, d1);
  // e1 = projectPointToLine(v00, v10, c)
  f2 ac2 = sub2(c, v00);
  f2 e1 = add2(v00, div2s(mul2s(q.ab2, dot2(q.ab2, ac2)), q.d22));
  float d0 = len2(sub2(c, e1)) / expectedWidth;
  return {sat(d0), sat(d1)};
}

// interpolateHairF32, swRasterizeHair.wgsl.ts:198-202
__device__ __forceinline__ float interpolateHairF32(f2 w, f4 v) {
  return mixf(mixf(v.x, v.y, w.x), mixf(v.z, v.w, w.x), w.y);
}

// projectHairPoint, swRasterizeHair.wgsl.ts:77-105
__device__ __forceinline__ void projectHairPoint(const float* modelMatrix, const float* vpMatrix,
                                                 f3 camPos, f4 pos, f4 tan, f2 size, float fiberRadius,
                                                 f2& o0, f2& o1, float& z0, float& z1) {
  f4 p0 = m4v(modelMatrix, mk4(pos.x, pos.y, pos.z, 1.0f));
  f4 t0 = m4v(modelMatrix, mk4(tan.x, tan.y, tan.z, 1.0f));
  f3 toCam = norm3(sub3(camPos, xyz(p0)));
  f3 right = mul3s(norm3(cross3(xyz(t0), toCam)), fiberRadius);
  f4 a = mk4(fsub(p0.x, right.x), fsub(p0.y, right.y), fsub(p0.z, right.z), 1.0f);
  f4 b = mk4(fadd(p0.x, right.x), fadd(p0.y, right.y), fadd(p0.z, right.z), 1.0f);
  f3 an = projectVertex(vpMatrix, a);
  f3 bn = projectVertex(vpMatrix, b);
  o0 = ndc2viewportPx(size, an);
  o1 = ndc2viewportPx(size, bn);
  z0 = an.z;
  z1 = bn.z;
}

__device__ __forceinline__ float loadTex2DClamp(const float* tex, uint32_t w, uint32_t h, int x, int y) {
  x = min(max(x, 0), (int)w - 1);
  y = min(max(y, 0), (int)h - 1);
  return __ldg(HFB_G(tex + (size_t)y * w + x));
}

}  // namespace hfb
