/*
 * TEST INFRASTRUCTURE -- the CPU oracle for the hair hot path.
 *
 * A serial C restatement of the reference's WGSL compute passes
 * (Scthe/frostbitten-hair-webgpu, src/passes/...).  It is used only by the
 * parity tests, by the smoke check and by the CPU-baseline leg of bench.py.
 * The product (libhairfb.so) never links, loads or calls anything here.
 *
 * Floating-point contract (shared with the CUDA kernels, which are an
 * independent implementation of the same WGSL):
 *   - every WGSL expression is evaluated left to right in fp32, one IEEE
 *     operation at a time, no fused multiply-add (built with
 *     -ffp-contract=off);
 *   - dot(a,b) = ((a.x*b.x + a.y*b.y) + a.z*b.z) [+ a.w*b.w];
 *     length(v) = sqrt(dot(v,v)); normalize(v) = v / length(v);
 *     mix(a,b,t) = a*(1-t) + b*t; fract(x) = x - floor(x);
 *     min/max = fminf/fmaxf; clamp(x,lo,hi) = min(max(x,lo),hi);
 *   - mat4 * vec4 (column-major) = ((c0*v.x + c1*v.y) + c2*v.z) + c3*v.w;
 *   - f32 -> u32 / i32 casts saturate and truncate toward zero, NaN -> 0
 *     (WGSL conversion rules);
 *   - the r32float 3D SDF texture with a linear/clamp-to-edge sampler is an
 *     exact fp32 trilinear filter with texel centres at (i + 0.5) / D;
 *   - out-of-range texel loads (depth, AO, shadow map) clamp to the edge;
 *   - pack2x16float rounds to nearest-even (overflow -> inf).
 *
 * Deterministic orders (the reference leaves these to atomic order):
 *   - tiles pass: segments are binned serially in (strand, segment) order,
 *     so every per-tile-depth-bin list is LIFO in that order;
 *   - tile sort: tiles enter their bucket in tile-index order;
 *   - fine pass: fragment slots inside one segment are allocated in pixel
 *     index order; pixels of a partial edge tile that lie outside the
 *     viewport take no part (they allocate nothing and count as done).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <assert.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* Types                                                                    */
/* ------------------------------------------------------------------------ */

typedef struct { float x, y; } v2;
typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;
typedef struct { float m[16]; } mat4;

/* Compile-time constants of the WGSL passes, see src/constants.ts:86-349.
 * Field order is part of the test harness ABI (oracle/oracle.py). */
typedef struct OracleConfig {
  uint32_t tileSize;                 /* CONFIG.hairRender.tileSize */
  uint32_t tileDepthBins;            /* CONFIG.hairRender.tileDepthBins */
  uint32_t slicesPerPixel;           /* CONFIG.hairRender.slicesPerPixel */
  uint32_t shadingPoints;            /* CONFIG.hairRender.shadingPoints */
  uint32_t gridDims;                 /* physicsForcesGrid.dims */
  uint32_t sortBuckets;              /* hairRender.sortBuckets */
  uint32_t sortBucketSize;           /* hairRender.sortBucketSize */
  uint32_t avgSegmentsPerTile;       /* hairRender.avgSegmentsPerTile */
  uint32_t avgFragmentsPerSlice;     /* hairRender.avgFragmentsPerSlice */
  uint32_t invalidTilesPerSegmentThreshold;
  uint32_t processorCount;           /* hairRender.processorCount */
  uint32_t alphaQuadratic;           /* hairRender.alphaQuadratic */
  float alphaMultiplier;             /* hairRender.alphaMultipler */
  float cameraNear, cameraFar;       /* camera.projection near/far */
  uint32_t reserved;
} OracleConfig;

/* struct Light / Shadows / AmbientOcclusion / HairMaterialParams / SDFCollider
 * / GridData / Uniforms: src/passes/renderUniformsBuffer.ts:46-137 */
typedef struct { v4 position; v4 colorAndEnergy; } OLight;
typedef struct {
  mat4 sourceModelViewMat, sourceProjMatrix, sourceMVP_Matrix;
  v4 sourcePosition;
  uint32_t usePCSS, PCF_Radius;
  float bias, strength;
} OShadows;
typedef struct {
  float radius, directionOffset, falloffStart2, falloffEnd2;
  uint32_t numDirections, numSteps;
  float strength, padding0;
} OAo;
typedef struct {
  float color0[3]; float specular;
  float color1[3]; float shadows;
  float weightTT, weightTRT, shift, roughness;
  float colorRng, lumaRng, attenuation, padding1;
} OHairMaterial;
typedef struct { v4 boundsMin, boundsMax; } OSdf;          /* sdfCollider.ts:10-23 */
typedef struct { v4 boundsMin; float boundsMax[3]; uint32_t debugDisplayValue; } OGridData; /* gridData.ts:17-21 */
typedef struct {
  mat4 vpMatrix, vpMatrixInv, viewMatrix, projMatrix, projMatrixInv;
  mat4 modelMatrix, modelViewMat, mvpMatrix, collisionSphereModelMatrix;
  v4 viewport, cameraPosition, colorMgmt, lightAmbient;
  OLight light0, light1, light2;
  OShadows shadows;
  OAo ao;
  OHairMaterial hairMaterial;
  OSdf sdf;
  OGridData gridData;
  float fiberRadius, dbgShadowMapPreviewSize;
  uint32_t maxDrawnHairSegments, displayMode;
  float background[8];
  float collisionSpherePosition[3];
  uint32_t gizmoActiveState;
} ORenderUniforms;
_Static_assert(sizeof(ORenderUniforms) == 1184, "Uniforms must be 1184 bytes");
_Static_assert(offsetof(ORenderUniforms, viewport) == 576, "viewport offset");
_Static_assert(offsetof(ORenderUniforms, shadows) == 736, "shadows offset");
_Static_assert(offsetof(ORenderUniforms, hairMaterial) == 992, "material offset");
_Static_assert(offsetof(ORenderUniforms, fiberRadius) == 1120, "fiberRadius offset");

/* struct SimulationUniforms: src/passes/simulation/simulationUniformsBuffer.ts:19-51 */
typedef struct {
  mat4 modelMatrix, modelMatrixInv;
  v4 collisionSphere, wind;
  OSdf sdf;
  OGridData gridData;
  float deltaTime, gravity; uint32_t constraintIterations, frameIdx;
  float windStrengthLull, windColisionTraceOffset, stiffnessLengthConstr, stiffnessCollisions;
  float stiffnessSDF, volumePreservation, friction, stiffnessGlobalConstr;
  float globalConstrExtent, globalConstrFade, stiffnessLocalConstr, windPhaseOffset;
  float windStrengthFrequency, windStrengthJitter, padding0, padding1;
} OSimUniforms;
_Static_assert(sizeof(OSimUniforms) == 304, "SimulationUniforms must be 304 bytes");
_Static_assert(offsetof(OSimUniforms, deltaTime) == 224, "deltaTime offset");

/* struct HairData: src/scene/hair/hairDataBuffer.ts:15-19 */
typedef struct { v4 boundingSphere; uint32_t strandsCount, pointsPerStrand; } OHairData;

/* ------------------------------------------------------------------------ */
/* Scalar / vector helpers (WGSL built-ins)                                 */
/* ------------------------------------------------------------------------ */

static inline float fmin_(float a, float b) { return fminf(a, b); }
static inline float fmax_(float a, float b) { return fmaxf(a, b); }
static inline float clampf_(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
static inline float sat(float x) { return clampf_(x, 0.0f, 1.0f); }
static inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline float fractf(float x) { return x - floorf(x); }
static inline uint32_t clampu(uint32_t x, uint32_t lo, uint32_t hi) {
  uint32_t r = x < lo ? lo : x;
  return r > hi ? hi : r;
}
/* WGSL u32(f32): saturating, toward zero, NaN -> 0 */
static inline uint32_t f2u(float f) {
  if (!(f > 0.0f)) return 0u;
  if (f >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)f;
}
/* WGSL i32(f32): saturating, toward zero, NaN -> 0 */
static inline int32_t f2i(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f <= -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

static inline v2 V2(float x, float y) { v2 r = {x, y}; return r; }
static inline v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v4 V4(float x, float y, float z, float w) { v4 r = {x, y, z, w}; return r; }
static inline v3 xyz(v4 a) { return V3(a.x, a.y, a.z); }

static inline v2 add2(v2 a, v2 b) { return V2(a.x + b.x, a.y + b.y); }
static inline v2 sub2(v2 a, v2 b) { return V2(a.x - b.x, a.y - b.y); }
static inline v2 mul2s(v2 a, float s) { return V2(a.x * s, a.y * s); }
static inline v2 div2s(v2 a, float s) { return V2(a.x / s, a.y / s); }
static inline float dot2(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
static inline float len2(v2 a) { return sqrtf(dot2(a, a)); }
static inline v2 norm2(v2 a) { float l = len2(a); return V2(a.x / l, a.y / l); }

static inline v3 add3(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 mul3s(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline v3 div3(v3 a, v3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline v3 div3s(v3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float len3(v3 a) { return sqrtf(dot3(a, a)); }
static inline v3 norm3(v3 a) { float l = len3(a); return V3(a.x / l, a.y / l, a.z / l); }
static inline v3 cross3(v3 a, v3 b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 mix3(v3 a, v3 b, float t) { return V3(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)); }
static inline v3 sat3(v3 a) { return V3(sat(a.x), sat(a.y), sat(a.z)); }
static inline v4 mix4(v4 a, v4 b, float t) {
  return V4(mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t), mixf(a.w, b.w, t));
}

static inline v4 m4v(const mat4* M, v4 v) {
  const float* m = M->m;
  v4 r;
  r.x = ((m[0] * v.x + m[4] * v.y) + m[8] * v.z) + m[12] * v.w;
  r.y = ((m[1] * v.x + m[5] * v.y) + m[9] * v.z) + m[13] * v.w;
  r.z = ((m[2] * v.x + m[6] * v.y) + m[10] * v.z) + m[14] * v.w;
  r.w = ((m[3] * v.x + m[7] * v.y) + m[11] * v.z) + m[15] * v.w;
  return r;
}

/* ------------------------------------------------------------------------ */
/* f16 helpers: pack2x16float / unpack2x16float                             */
/* ------------------------------------------------------------------------ */

static uint16_t f32_to_f16_rne(float f) {
  uint32_t x; memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t e = (x >> 23) & 0xFFu;
  uint32_t m = x & 0x7FFFFFu;
  if (e == 0xFFu) return (uint16_t)(sign | 0x7C00u | (m ? 0x200u : 0u));
  int32_t E = (int32_t)e - 127 + 15;
  if (E >= 31) return (uint16_t)(sign | 0x7C00u);
  if (E <= 0) {
    if (E < -10) return (uint16_t)sign;
    m |= 0x800000u;
    uint32_t shift = (uint32_t)(14 - E);
    uint32_t hm = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1u);
    if (rem > half || (rem == half && (hm & 1u))) hm++;
    return (uint16_t)(sign | hm);
  }
  uint32_t hm = m >> 13;
  uint32_t rem = m & 0x1FFFu;
  uint32_t h = sign | ((uint32_t)E << 10) | hm;
  if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u))) h++;
  return (uint16_t)h;
}

static float f16_to_f32(uint16_t h) {
  uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
  uint32_t e = ((uint32_t)h >> 10) & 0x1Fu;
  uint32_t m = (uint32_t)h & 0x3FFu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) x = sign;
    else {
      int32_t E = -1;
      do { E++; m <<= 1; } while (!(m & 0x400u));
      m &= 0x3FFu;
      x = sign | ((uint32_t)(127 - 15 - E) << 23) | (m << 13);
    }
  } else if (e == 31) {
    x = sign | 0x7F800000u | (m << 13);
  } else {
    x = sign | ((e - 15 + 127) << 23) | (m << 13);
  }
  float f; memcpy(&f, &x, 4);
  return f;
}

EXPORT uint16_t oracle_f32_to_f16(float f) { return f32_to_f16_rne(f); }
EXPORT float oracle_f16_to_f32(uint16_t h) { return f16_to_f32(h); }

/* ------------------------------------------------------------------------ */
/* GENERIC_UTILS: src/passes/_shaderSnippets/shaderSnippets.wgls.ts:61-166  */
/* ------------------------------------------------------------------------ */

#define FLOAT_EPSILON 1e-7f
static const float PI_F = 3.141592653589793f;

/* projectVertex, shaderSnippets.wgls.ts:92-96 */
static inline v3 projectVertex(const mat4* mvp, v4 pos) {
  v4 c = m4v(mvp, pos);
  return V3(c.x / c.w, c.y / c.w, c.z / c.w);
}

/* projectPointToLine, shaderSnippets.wgls.ts:99-105 */
static inline v2 projectPointToLine(v2 l1, v2 l2, v2 p) {
  v2 ab = sub2(l2, l1);
  v2 ac = sub2(p, l1);
  float d1 = dot2(ab, ac);
  float d2 = dot2(ab, ab);
  v2 ad = div2s(mul2s(ab, d1), d2);
  return add2(l1, ad);
}

/* ndc2viewportPx, shaderSnippets.wgls.ts:107-110 */
static inline v2 ndc2viewportPx(v2 size, v3 pos) {
  v2 p01 = V2(pos.x * 0.5f + 0.5f, pos.y * 0.5f + 0.5f);
  return V2(p01.x * size.x, p01.y * size.y);
}

/* remapToIndices, shaderSnippets.wgls.ts:124-130 */
static inline float remapToIndices(uint32_t maxIdx, float t, uint32_t* i0, uint32_t* i1) {
  float a = t * ((float)maxIdx - 1.0f);
  uint32_t au = f2u(a);
  *i0 = clampu(au, 0u, maxIdx - 1u);
  *i1 = clampu(au + 1u, 0u, maxIdx - 1u);
  return fractf(a);
}

/* toLuma_fromLinear, shaderSnippets.wgls.ts:133-136 */
static inline float toLuma(v3 c) { return dot3(V3(0.2126729f, 0.7151522f, 0.0721750f), c); }

/* getDepthBin, shaderSnippets.wgls.ts:152-160 */
static inline uint32_t getDepthBin(uint32_t binCount, v2 tileDepth, float pixelDepth) {
  float span = fabsf(tileDepth.y - tileDepth.x);
  float t = (pixelDepth - tileDepth.x) / span;
  return clampu(f2u(t * (float)binCount), 0u, binCount - 1u);
}

/* randomRGB, src/passes/_shaderSnippets/noise.wgsl.ts:45-51 */
static inline v3 randomRGB(uint32_t v, float b) {
  float fv = (float)v;
  return sat3(V3(fractf(fv * 1.73f) * b, fractf(fv * 1.17f) * b, fractf(fv * 1.31f) * b));
}

/* FresnelSchlick1, src/passes/_shaderSnippets/pbr.wgsl.ts:22-24 */
static inline float FresnelSchlick1(float c, float F0) {
  return F0 + (1.0f - F0) * powf(1.0f - c, 5.0f);
}

/* ------------------------------------------------------------------------ */
/* SW raster utils: src/passes/swHair/shaderImpl/swRasterizeHair.wgsl.ts    */
/* ------------------------------------------------------------------------ */

typedef struct { v2 v00, v01, v10, v11; v4 depthsProj; } ProjSeg;

/* projectHairPoint, swRasterizeHair.wgsl.ts:77-105 */
static void projectHairPoint(const ORenderUniforms* U, const float* pos, const float* tan,
                             uint32_t P, uint32_t strand, uint32_t point, v2 size, float fiberRadius,
                             v2* o0, v2* o1, v2* depths) {
  const float* p = pos + 4u * ((size_t)strand * P + point);
  const float* t = tan + 4u * ((size_t)strand * P + point);
  v4 p0 = m4v(&U->modelMatrix, V4(p[0], p[1], p[2], 1.0f));
  v4 t0 = m4v(&U->modelMatrix, V4(t[0], t[1], t[2], 1.0f));
  v3 toCam = norm3(sub3(xyz(U->cameraPosition), xyz(p0)));
  v3 right = mul3s(norm3(cross3(xyz(t0), toCam)), fiberRadius);
  v4 a = V4(p0.x - right.x, p0.y - right.y, p0.z - right.z, 1.0f);
  v4 b = V4(p0.x + right.x, p0.y + right.y, p0.z + right.z, 1.0f);
  v3 an = projectVertex(&U->vpMatrix, a);
  v3 bn = projectVertex(&U->vpMatrix, b);
  *o0 = ndc2viewportPx(size, an);
  *o1 = ndc2viewportPx(size, bn);
  *depths = V2(an.z, bn.z);
}

/* projectHairSegment, swRasterizeHair.wgsl.ts:39-68 */
static ProjSeg projectHairSegment(const ORenderUniforms* U, const float* pos, const float* tan,
                                  uint32_t P, uint32_t strand, uint32_t seg, v2 size, float fr) {
  ProjSeg r; v2 d;
  projectHairPoint(U, pos, tan, P, strand, seg, size, fr, &r.v00, &r.v01, &d);
  r.depthsProj.x = d.x; r.depthsProj.y = d.y;
  projectHairPoint(U, pos, tan, P, strand, seg + 1u, size, fr, &r.v10, &r.v11, &d);
  r.depthsProj.z = d.x; r.depthsProj.w = d.y;
  return r;
}

/* getRasterizedHairBounds, swRasterizeHair.wgsl.ts:111-124 */
static v4 getRasterizedHairBounds(const ProjSeg* r, v2 size) {
  float mx = ceilf(fmax_(fmax_(r->v00.x, r->v01.x), fmax_(r->v10.x, r->v11.x)));
  float my = ceilf(fmax_(fmax_(r->v00.y, r->v01.y), fmax_(r->v10.y, r->v11.y)));
  float nx = floorf(fmin_(fmin_(r->v00.x, r->v01.x), fmin_(r->v10.x, r->v11.x)));
  float ny = floorf(fmin_(fmin_(r->v00.y, r->v01.y), fmin_(r->v10.y, r->v11.y)));
  mx = fmin_(mx, size.x); my = fmin_(my, size.y);
  nx = fmax_(nx, 0.0f); ny = fmax_(ny, 0.0f);
  return V4(nx, ny, mx, my);
}

/* edgeFunction, swRasterizeHair.wgsl.ts:128-130 */
static inline float edgeFunction(v2 v0, v2 v1, v2 p) {
  return (p.x - v0.x) * (v1.y - v0.y) - (p.y - v0.y) * (v1.x - v0.x);
}

/* debugBarycentric, swRasterizeHair.wgsl.ts:150-159 */
static inline uint32_t debugBarycentric(v4 w) {
  uint32_t c0 = f2u(sat(w.x) * 255.0f);
  uint32_t c1 = f2u(sat(w.y) * 255.0f);
  uint32_t c2 = f2u(sat(w.z) * 255.0f);
  return 0xff000000u | c0 | (c1 << 8) | (c2 << 16);
}

/* interpolateHairQuad, swRasterizeHair.wgsl.ts:170-196 */
static v2 interpolateHairQuad(const ProjSeg* s, v2 c) {
  v2 sm = div2s(add2(s->v00, s->v01), 2.0f);
  v2 em = div2s(add2(s->v10, s->v11), 2.0f);
  v2 cp = projectPointToLine(sm, em, c);
  float d1 = len2(sub2(cp, sm)) / len2(sub2(sm, em));
  float widthStart = len2(sub2(s->v00, s->v01));
  float widthEnd = widthStart * dot2(norm2(sub2(s->v00, s->v01)), norm2(sub2(s->v10, s->v11)));
  float expectedWidth = mixf(widthStart, widthEnd, d1);
  v2 e1 = projectPointToLine(s->v00, s->v10, c);
  float d0 = len2(sub2(c, e1)) / expectedWidth;
  return V2(sat(d0), sat(d1));
}

/* interpolateHairF32, swRasterizeHair.wgsl.ts:198-202 */
static inline float interpolateHairF32(v2 w, v4 v) {
  float a = mixf(v.x, v.y, w.x);
  float b = mixf(v.z, v.w, w.x);
  return mixf(a, b, w.y);
}

/* ------------------------------------------------------------------------ */
/* Texture loads with clamp-to-edge                                         */
/* ------------------------------------------------------------------------ */

static inline float loadTex2D(const float* tex, uint32_t w, uint32_t h, int64_t x, int64_t y) {
  if (x < 0) x = 0;
  if (y < 0) y = 0;
  if (x > (int64_t)w - 1) x = (int64_t)w - 1;
  if (y > (int64_t)h - 1) y = (int64_t)h - 1;
  return tex[(size_t)y * w + (size_t)x];
}

/* ------------------------------------------------------------------------ */
/* SW raster golden test shader: src/passes/swHair/swRasterizer.test.ts:186-248 */
/* ------------------------------------------------------------------------ */

EXPORT void oracle_sw_raster_test(const void* uniforms, const void* hairData,
                                  const float* positions, const float* tangents,
                                  uint32_t* result /* W*H u32, zero-initialised */) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  const OHairData* H = (const OHairData*)hairData;
  v2 size = V2(U->viewport.x, U->viewport.y);
  uint32_t W = f2u(size.x), Hh = f2u(size.y);
  uint32_t P = H->pointsPerStrand;
  for (uint32_t strand = 0; strand < H->strandsCount; strand++) {
    for (uint32_t seg = 0; seg + 1u < P; seg++) {
      ProjSeg s = projectHairSegment(U, positions, tangents, P, strand, seg, size, U->fiberRadius);
      v4 b = getRasterizedHairBounds(&s, size);
      for (float y = b.y; y < b.w; y += 1.0f) {
        for (float x = b.x; x < b.z; x += 1.0f) {
          v2 p = V2(x, y);
          float C0 = edgeFunction(s.v01, s.v00, p);
          float C1 = edgeFunction(s.v11, s.v01, p);
          float C2 = edgeFunction(s.v10, s.v11, p);
          float C3 = edgeFunction(s.v00, s.v10, p);
          if (C0 >= 0 && C1 >= 0 && C2 >= 0 && C3 >= 0) {
            v2 w = interpolateHairQuad(&s, p);
            uint32_t value = debugBarycentric(V4(w.x, w.y, 0.1f, 0.0f));
            uint32_t px = f2u(x), py = f2u(y);
            if (px >= W || py >= Hh) continue;
            uint32_t row = Hh - py;
            size_t idx = (size_t)row * W + px;
            if (idx >= (size_t)W * Hh) continue; /* robust access: dropped */
            if (value > result[idx]) result[idx] = value;
          }
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Tile utils: src/passes/swHair/shaderImpl/tileUtils.wgsl.ts:5-54          */
/* ------------------------------------------------------------------------ */

static inline uint32_t divCeil(uint32_t a, uint32_t b) { return (a + b - 1u) / b; }

typedef struct { uint32_t x0, y0, x1, y1; } TileBounds;

/* getTileBoundsPx, tileUtils.wgsl.ts:43-54 (with scissorWithViewport) */
static inline TileBounds getTileBoundsPx(uint32_t W, uint32_t H, uint32_t TS, uint32_t tx, uint32_t ty) {
  TileBounds b;
  b.x0 = clampu(tx * TS, 0u, W - 1u);
  b.y0 = clampu(ty * TS, 0u, H - 1u);
  b.x1 = clampu((tx + 1u) * TS, 0u, W - 1u);
  b.y1 = clampu((ty + 1u) * TS, 0u, H - 1u);
  return b;
}

/* ------------------------------------------------------------------------ */
/* HairTilesPass: src/passes/swHair/hairTilesPass.wgsl.ts:70-246            */
/* ------------------------------------------------------------------------ */

#define MAX_U32 0xffffffffu
#define INVALID_PTR 0xffffffffu

/*
 * tilesBuf:   T*B entries of {minDepth, maxDepth, tileSegmentPtr, pad} (u32),
 *             zero-initialised by the caller (cmdClearBeforeRender).
 * segBuf:     u32 drawnSegmentsCount followed by maxDrawnSegments entries of
 *             {strandAndSegmentIdxs, next}; the counter must be zeroed.
 * segCount:   T u32 counters, zero-initialised.
 */
EXPORT void oracle_tiles_pass(const OracleConfig* cfg, const void* uniforms, const void* hairData,
                              const float* positions, const float* tangents,
                              const float* depth /* W*H, texel row 0 = top */,
                              uint32_t strandsToRender,
                              uint32_t* tilesBuf, uint32_t* segBuf, uint32_t* segCount) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  const OHairData* HD = (const OHairData*)hairData;
  v2 size = V2(U->viewport.x, U->viewport.y);
  uint32_t W = f2u(size.x), H = f2u(size.y);
  uint32_t TS = cfg->tileSize, B = cfg->tileDepthBins;
  uint32_t tilesX = divCeil(W, TS);
  uint32_t maxDrawn = U->maxDrawnHairSegments;
  uint32_t P = HD->pointsPerStrand;
  uint32_t S = HD->strandsCount;
  const float fMAX_U32 = (float)MAX_U32;

  /* getHairDepthBoundsVS, hairTilesPass.wgsl.ts:242-246 */
  v4 bs = HD->boundingSphere;
  v4 bsVS = m4v(&U->modelViewMat, V4(bs.x, bs.y, bs.z, 1.0f));
  v2 depthBoundsVS = V2(bsVS.z - bs.w, bsVS.z + bs.w);

  uint32_t nStrands = strandsToRender < S ? strandsToRender : S;
  /* Phase 1 (parallel over strands, static contiguous ranges): every
   * (segment, tile) that passes becomes a record, appended in canonical
   * (strand, segment, tileY, tileX) order inside each thread's range. */
  typedef struct { uint32_t strand, seg, tx, ty, bin; float dmin, dmax; } Rec;
  int nth = 1;
#ifdef _OPENMP
  nth = omp_get_max_threads();
#endif
  Rec** recs = (Rec**)calloc((size_t)nth, sizeof(Rec*));
  size_t* nrec = (size_t*)calloc((size_t)nth, sizeof(size_t));
  size_t* caprec = (size_t*)calloc((size_t)nth, sizeof(size_t));
#pragma omp parallel num_threads(nth)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    uint32_t lo = (uint32_t)(((uint64_t)nStrands * (uint64_t)tid) / (uint64_t)nth);
    uint32_t hi = (uint32_t)(((uint64_t)nStrands * (uint64_t)(tid + 1)) / (uint64_t)nth);
    for (uint32_t strand = lo; strand < hi; strand++) {
      for (uint32_t seg = 0; seg + 1u < P; seg++) {
        ProjSeg s = projectHairSegment(U, positions, tangents, P, strand, seg, size, U->fiberRadius);
        v4 b = getRasterizedHairBounds(&s, size);
        uint32_t tminx = f2u(b.x) / TS, tminy = f2u(b.y) / TS;
        uint32_t tmaxx = f2u(b.z) / TS, tmaxy = f2u(b.w) / TS;
        uint32_t tsx = (tmaxx - tminx) + 1u, tsy = (tmaxy - tminy) + 1u;
        if (tsx * tsy > cfg->invalidTilesPerSegmentThreshold) continue;
        for (uint32_t ty = tminy; ty <= tmaxy; ty++) {
          for (uint32_t tx = tminx; tx <= tmaxx; tx++) {
            /* processTile, hairTilesPass.wgsl.ts:139-238 */
            TileBounds tb = getTileBoundsPx(W, H, TS, tx, ty);
            float dmin = 999.0f, dmax = -999.0f;
            uint32_t dbin = B;
            for (uint32_t y = tb.y0; y < tb.y1; y++) {
              for (uint32_t x = tb.x0; x < tb.x1; x++) {
                v2 p = V2((float)x, (float)y);
                float C0 = edgeFunction(s.v01, s.v00, p);
                float C1 = edgeFunction(s.v11, s.v01, p);
                float C2 = edgeFunction(s.v10, s.v11, p);
                float C3 = edgeFunction(s.v00, s.v10, p);
                if (C0 >= 0 && C1 >= 0 && C2 >= 0 && C3 >= 0) {
                  v2 w = interpolateHairQuad(&s, p);
                  float hd = interpolateHairF32(w, s.depthsProj);
                  float zb = loadTex2D(depth, W, H, (int64_t)x, (int64_t)H - (int64_t)y);
                  if (hd > zb) continue;
                  v3 vs = projectVertex(&U->projMatrixInv, V4(p.x, p.y, hd, 1.0f));
                  uint32_t bin = (B - 1u) - getDepthBin(B, depthBoundsVS, vs.z);
                  dmin = fmin_(dmin, hd);
                  dmax = fmax_(dmax, hd);
                  dbin = dbin < bin ? dbin : bin;
                }
              }
            }
            if (dmin > 1.0f) continue;
            if (nrec[tid] == caprec[tid]) {
              caprec[tid] = caprec[tid] ? 2 * caprec[tid] : 1024;
              recs[tid] = (Rec*)realloc(recs[tid], caprec[tid] * sizeof(Rec));
            }
            Rec r = {strand, seg, tx, ty, dbin, dmin, dmax};
            recs[tid][nrec[tid]++] = r;
          }
        }
      }
    }
  }
  /* Phase 2 (serial): allocate pointers and link the lists in canonical
   * order, as one serial dispatch of the WGSL would. */
  for (int t = 0; t < nth; t++) {
    for (size_t i = 0; i < nrec[t]; i++) {
      const Rec* r = &recs[t][i];
      uint32_t nextPtr = segBuf[0]++;
      if (nextPtr < maxDrawn) {
        /* _storeTileHead, hairTilesResultBuffer.ts:14-42 */
        uint32_t ti = r->ty * tilesX * B + r->tx * B + r->bin;
        uint32_t dmaxU = f2u(r->dmax * fMAX_U32);
        uint32_t dminU = f2u((1.0f - r->dmin) * fMAX_U32);
        uint32_t* head = tilesBuf + 4u * (size_t)ti;
        if (dminU > head[0]) head[0] = dminU;
        if (dmaxU > head[1]) head[1] = dmaxU;
        uint32_t last = head[2];
        head[2] = nextPtr + 1u;
        uint32_t prevPtr = last == 0u ? INVALID_PTR : last - 1u;
        /* _storeTileSegment, hairTileSegmentsBuffer.ts:22-29 */
        segBuf[1u + 2u * (size_t)nextPtr] = (r->seg << 24) | r->strand;
        segBuf[2u + 2u * (size_t)nextPtr] = prevPtr;
        /* _incTileSegmentCount, segmentCountPerTileBuffer.ts:21-26 */
        segCount[r->ty * tilesX + r->tx] += 1u;
      }
    }
    free(recs[t]);
  }
  free(recs); free(nrec); free(caprec);
}

/* ------------------------------------------------------------------------ */
/* HairTileSortPass: hairTileSortPass.countTiles.wgsl.ts:21-97 and          */
/* hairTileSortPass.sort.wgsl.ts:35-75                                      */
/* ------------------------------------------------------------------------ */

/* buckets: sortBuckets * {tileCount, writeOffset}; tileList: {drawnTiles, data[T]}.
 * Both zero-initialised by the caller (cmdClearBeforeRender). */
EXPORT void oracle_tile_sort(const OracleConfig* cfg, uint32_t W, uint32_t H,
                             const uint32_t* segCount, uint32_t* buckets, uint32_t* tileList) {
  uint32_t TS = cfg->tileSize;
  uint32_t T = divCeil(W, TS) * divCeil(H, TS);
  uint32_t NB = cfg->sortBuckets;
  /* count-tiles */
  for (uint32_t t = 0; t < T; t++) {
    uint32_t c = segCount[t];
    if (c > 0u) {
      uint32_t k = clampu(c / cfg->sortBucketSize, 0u, NB - 1u);
      buckets[2u * k] += 1u;
    }
  }
  /* calculateOffsetsForEachBucket: reverse exclusive scan, heavy first */
  uint32_t* offs = (uint32_t*)calloc(NB, sizeof(uint32_t));
  uint32_t off = 0;
  for (uint32_t i = 0; i < NB; i++) {
    uint32_t idx = NB - 1u - i;
    offs[idx] = off;
    off += buckets[2u * idx];
  }
  for (uint32_t t = 0; t < T; t++) {
    uint32_t c = segCount[t];
    if (c > 0u) {
      uint32_t k = clampu(c / cfg->sortBucketSize, 0u, NB - 1u);
      uint32_t inBucket = buckets[2u * k + 1u]++;
      tileList[1u + offs[k] + inBucket] = t;
      tileList[0] += 1u;
    }
  }
  free(offs);
}

/* ------------------------------------------------------------------------ */
/* HairFinePass: src/passes/swHair/hairFinePass.wgsl.ts:126-335,            */
/* processHairSegment.wgsl.ts:5-70, reduceHairSlices.wgsl.ts:9-78           */
/* ------------------------------------------------------------------------ */

#define ALPHA_CUTOFF 0.999f

/* _sampleShading, src/scene/hair/hairShadingBuffer.ts:28-38 */
static inline v4 sampleShading(const float* shading, uint32_t SP, uint32_t strand, float t) {
  uint32_t i0, i1;
  float f = remapToIndices(SP, t, &i0, &i1);
  const float* c0 = shading + 4u * ((size_t)strand * SP + i0);
  const float* c1 = shading + 4u * ((size_t)strand * SP + i1);
  return mix4(V4(c0[0], c0[1], c0[2], c0[3]), V4(c1[0], c1[1], c1[2], c1[3]), f);
}

typedef struct { uint16_t c[4]; uint32_t next; } SliceEntry;

/*
 * result: 4 u32/f32 header (the first u32 is tileQueueAtomicIdx) followed by
 * W*H vec4f, zero-initialised by the caller (cmdClearBeforeRender).
 */
EXPORT void oracle_fine_pass(const OracleConfig* cfg, const void* uniforms, const void* hairData,
                             const float* positions, const float* tangents, const float* shading,
                             const float* depth, const uint32_t* tilesBuf, const uint32_t* segBuf,
                             const uint32_t* tileList, float* result) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  const OHairData* HD = (const OHairData*)hairData;
  v2 size = V2(U->viewport.x, U->viewport.y);
  uint32_t W = f2u(size.x), H = f2u(size.y);
  uint32_t TS = cfg->tileSize, B = cfg->tileDepthBins, L = cfg->slicesPerPixel;
  uint32_t SP = cfg->shadingPoints;
  uint32_t tilesX = divCeil(W, TS), tilesY = divCeil(H, TS);
  uint32_t tileCount = tilesX * tilesY;
  uint32_t P = HD->pointsPerStrand;
  uint32_t maxDrawn = U->maxDrawnHairSegments;
  uint32_t maxProcessed = HD->strandsCount * P;
  uint32_t NPX = TS * TS;
  uint32_t CAP = cfg->avgFragmentsPerSlice * L * TS * TS; /* SLICE_DATA_PER_PROCESSOR_COUNT */
  const float fMAX_U32 = (float)MAX_U32;
  /* getDbgSlicesModeMaxSlices, renderUniformsBuffer.ts:144-146 */
  uint32_t dispMode = U->displayMode & 0xffu;
  uint32_t dbgMax = dispMode == 4u ? ((U->displayMode >> 8) & 0xffffu) : 0u;
  int isDbg = dbgMax != 0u;

  float* res = result + 4;
  uint32_t drawnTiles = tileList[0];
  /* tiles are independent (each writes only its own pixels): any order and
   * any number of processors give the same result */
#pragma omp parallel
  {
  SliceEntry* pool = (SliceEntry*)malloc(sizeof(SliceEntry) * (size_t)CAP);
  uint32_t* heads = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)NPX * L);
  uint8_t* done = (uint8_t*)malloc(NPX);
#pragma omp for schedule(dynamic, 1)
  for (uint32_t q = 0; q < drawnTiles; q++) {
    uint32_t tileIdx = tileList[1u + q];
    if (tileIdx >= tileCount) continue;
    uint32_t tx = tileIdx % tilesX, ty = tileIdx / tilesX;
    TileBounds tbp = getTileBoundsPx(W, H, TS, tx, ty);
    for (uint32_t i = 0; i < NPX * L; i++) heads[i] = INVALID_PTR;
    for (uint32_t p = 0; p < NPX; p++) {
      uint32_t px = tbp.x0 + p % TS, py = tbp.y0 + p / TS;
      done[p] = (px >= W || py >= H) ? 1 : 0; /* outside the viewport: inactive */
    }

    for (uint32_t bin = 0; bin < B; bin++) {
      uint32_t ti = ty * tilesX * B + tx * B + bin;
      const uint32_t* head = tilesBuf + 4u * (size_t)ti;
      /* _getTileDepth, hairTilesResultBuffer.ts:47-54 */
      v2 tileDepth = V2((float)(MAX_U32 - head[0]) / fMAX_U32, (float)head[1] / fMAX_U32);
      if (tileDepth.y != 0.0f) {
        uint32_t segPtr = head[2] == 0u ? INVALID_PTR : head[2] - 1u;
        uint32_t sliceOff = 0;
        uint32_t processed = 0;
        while (processed < maxProcessed) {
          if (segPtr >= maxDrawn || segPtr == INVALID_PTR) { sliceOff = CAP; break; }
          uint32_t enc = segBuf[1u + 2u * (size_t)segPtr];
          uint32_t strand = enc & 0x00ffffffu, seg = enc >> 24;
          uint32_t nextPtr = segBuf[2u + 2u * (size_t)segPtr];
          ProjSeg s = projectHairSegment(U, positions, tangents, P, strand, seg, size, U->fiberRadius);
          for (uint32_t p = 0; p < NPX; p++) {
            if (done[p]) continue;
            /* processHairSegment, processHairSegment.wgsl.ts:5-54 */
            v2 pos = V2((float)(tbp.x0 + p % TS), (float)(tbp.y0 + p / TS));
            float C0 = edgeFunction(s.v01, s.v00, pos);
            float C1 = edgeFunction(s.v11, s.v01, pos);
            float C2 = edgeFunction(s.v10, s.v11, pos);
            float C3 = edgeFunction(s.v00, s.v10, pos);
            if (C0 < 0 || C1 < 0 || C2 < 0 || C3 < 0) continue;
            v2 w = interpolateHairQuad(&s, pos);
            float t = w.y;
            float hd = interpolateHairF32(w, s.depthsProj);
            float zb = loadTex2D(depth, W, H, (int64_t)f2i(pos.x), (int64_t)f2i(size.y - pos.y));
            if (hd >= zb) continue;
            uint32_t slot = sliceOff++;
            if (slot >= CAP) continue;
            /* getAlphaCoverage, processHairSegment.wgsl.ts:60-69 */
            float alpha = 1.0f - fabsf(w.x * 2.0f - 1.0f);
            if (cfg->alphaQuadratic) alpha = sqrtf(alpha);
            alpha = sat(alpha * cfg->alphaMultiplier);
            float tFull = ((float)seg + t) / (float)(P - 1u);
            v4 color = sampleShading(shading, SP, strand, tFull);
            color.w = color.w * alpha;
            /* getSliceIdx */
            uint32_t sl = getDepthBin(L, tileDepth, hd);
            uint32_t prev = heads[p * L + sl];
            heads[p * L + sl] = slot;
            pool[slot].c[0] = f32_to_f16_rne(color.x);
            pool[slot].c[1] = f32_to_f16_rne(color.y);
            pool[slot].c[2] = f32_to_f16_rne(color.z);
            pool[slot].c[3] = f32_to_f16_rne(color.w);
            pool[slot].next = prev;
          }
          if (sliceOff >= CAP) break;
          processed++;
          segPtr = nextPtr;
        }
        if (sliceOff != 0u) {
          for (uint32_t p = 0; p < NPX; p++) {
            if (done[p]) continue;
            uint32_t px = tbp.x0 + p % TS, py = tbp.y0 + p / TS;
            /* reduceHairSlices, reduceHairSlices.wgsl.ts:9-73 */
            float* dst = res + 4u * ((size_t)W * py + px);
            float fr = dst[0], fg = dst[1], fb = dst[2], fa = dst[3];
            uint32_t sliceCount = isDbg ? f2u(fr * (float)dbgMax) : 0u;
            uint32_t s = 0;
            for (; s < L; s++) {
              if (!isDbg && fa >= ALPHA_CUTOFF) break;
              uint32_t ptr = heads[p * L + s];
              while (ptr != INVALID_PTR && ptr < CAP) {
                if (!isDbg && fa >= ALPHA_CUTOFF) break;
                const SliceEntry* e = &pool[ptr];
                ptr = e->next;
                sliceCount += 1u;
                float k = 1.0f - fa;
                fr = fr + f16_to_f32(e->c[0]) * k;
                fg = fg + f16_to_f32(e->c[1]) * k;
                fb = fb + f16_to_f32(e->c[2]) * k;
                fa = fa + f16_to_f32(e->c[3]) * k;
              }
              heads[p * L + s] = INVALID_PTR;
            }
            for (; s < L; s++) heads[p * L + s] = INVALID_PTR;
            if (isDbg) {
              float c = sat((float)sliceCount / (float)dbgMax);
              fr = c; fg = 0.0f; fb = 0.0f; fa = 1.0f;
            }
            dst[0] = fr; dst[1] = fg; dst[2] = fb; dst[3] = fa;
            done[p] = (!isDbg && fa >= ALPHA_CUTOFF) ? 1 : 0;
          }
        }
      }
      /* checkAllPixelsInWkgrpDone, hairFinePass.wgsl.ts:305-327 */
      int all = 1;
      for (uint32_t p = 0; p < NPX; p++) if (!done[p]) { all = 0; break; }
      if (all) break;
    }
  }
  free(pool); free(heads); free(done);
  }
  result[0] = 0.0f; /* the tile queue counter is not modelled */
}

/* ------------------------------------------------------------------------ */
/* Grids: src/passes/simulation/grids/grids.wgsl.ts:3-92 and the two grid   */
/* buffers densityVelocityGrid.wgsl.ts / densityGradAndWindGrid.wgsl.ts     */
/* ------------------------------------------------------------------------ */

#define GRID_FLOAT_TO_U32_MUL 1000000.0f

static inline int32_t gridEncode(float v) { return f2i(v * GRID_FLOAT_TO_U32_MUL); }
static inline float gridDecode(int32_t v) { return (float)v / GRID_FLOAT_TO_U32_MUL; }

static inline uint32_t gridIdx(uint32_t G, uint32_t x, uint32_t y, uint32_t z) {
  return clampu(z, 0u, G - 1u) * G * G + clampu(y, 0u, G - 1u) * G + clampu(x, 0u, G - 1u);
}

typedef struct { uint32_t mn[3], mx[3]; v3 pInGrid; } GridCo;

/* _getGridCell, grids.wgsl.ts:43-56 */
static inline GridCo getGridCell(uint32_t G, v3 bmin, v3 bmax, v3 p) {
  v3 t = sat3(div3(sub3(p, bmin), sub3(bmax, bmin)));
  float g = (float)(G - 1u);
  GridCo r;
  r.pInGrid = mul3s(t, g);
  v3 a = mul3s(t, g);
  r.mn[0] = f2u(floorf(a.x)); r.mn[1] = f2u(floorf(a.y)); r.mn[2] = f2u(floorf(a.z));
  r.mx[0] = f2u(ceilf(a.x)); r.mx[1] = f2u(ceilf(a.y)); r.mx[2] = f2u(ceilf(a.z));
  return r;
}

/* _getGridCellWeights, grids.wgsl.ts:58-66 */
static inline v3 cellWeights(uint32_t x, uint32_t y, uint32_t z, v3 p) {
  return V3(clampf_(1.0f - fabsf(p.x - (float)x), 0.0f, 1.0f),
            clampf_(1.0f - fabsf(p.y - (float)y), 0.0f, 1.0f),
            clampf_(1.0f - fabsf(p.z - (float)z), 0.0f, 1.0f));
}

/* _getGridDensityVelocity, densityVelocityGrid.wgsl.ts:35-73 */
static void gatherDensityVelocity(uint32_t G, const int32_t* grid, v3 bmin, v3 bmax, v3 p,
                                  v3* vel, float* dens) {
  GridCo co = getGridCell(G, bmin, bmax, p);
  v3 rv = V3(0, 0, 0); float rd = 0.0f;
  for (uint32_t z = co.mn[2]; z <= co.mx[2]; z++)
    for (uint32_t y = co.mn[1]; y <= co.mx[1]; y++)
      for (uint32_t x = co.mn[0]; x <= co.mx[0]; x++) {
        v3 w = cellWeights(x, y, z, co.pInGrid);
        const int32_t* c = grid + 4u * gridIdx(G, x, y, z);
        v3 v = V3(gridDecode(c[0]), gridDecode(c[1]), gridDecode(c[2]));
        float d = gridDecode(c[3]);
        rv = add3(rv, mul3(w, v));
        rd = rd + len3(w) * d;
      }
  *vel = rv; *dens = rd;
}

/* _getGridDensityGradAndWind, densityGradAndWindGrid.wgsl.ts:20-44 */
static void gatherGradWind(uint32_t G, const float* grid, v3 bmin, v3 bmax, v3 p, v3* grad, float* wind) {
  GridCo co = getGridCell(G, bmin, bmax, p);
  v3 rg = V3(0, 0, 0); float rw = 0.0f;
  for (uint32_t z = co.mn[2]; z <= co.mx[2]; z++)
    for (uint32_t y = co.mn[1]; y <= co.mx[1]; y++)
      for (uint32_t x = co.mn[0]; x <= co.mx[0]; x++) {
        v3 w = cellWeights(x, y, z, co.pInGrid);
        const float* c = grid + 4u * gridIdx(G, x, y, z);
        rg = add3(rg, mul3(w, V3(c[0], c[1], c[2])));
        rw = rw + len3(w) * c[3];
      }
  *grad = rg; *wind = rw;
}

/* sampleSDFCollider, src/scene/sdfCollider/sdfCollider.ts:36-44 with the
 * linear / clamp-to-edge sampler of sdfUtils.ts:33-42 */
static float sampleSDF(const float* sdf, uint32_t D, v3 bmin, v3 bmax, v3 p) {
  v3 t = sat3(div3(sub3(p, bmin), sub3(bmax, bmin)));
  float fD = (float)D;
  float u = t.x * fD - 0.5f, v = t.y * fD - 0.5f, w = t.z * fD - 0.5f;
  float fu = floorf(u), fv = floorf(v), fw = floorf(w);
  float ax = u - fu, ay = v - fv, az = w - fw;
  int32_t x0 = (int32_t)fu, y0 = (int32_t)fv, z0 = (int32_t)fw;
  int32_t x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
  int32_t m = (int32_t)D - 1;
#define CL(a) ((a) < 0 ? 0 : ((a) > m ? m : (a)))
  x0 = CL(x0); x1 = CL(x1); y0 = CL(y0); y1 = CL(y1); z0 = CL(z0); z1 = CL(z1);
#undef CL
#define T(x, y, z) sdf[((size_t)(z) * D + (size_t)(y)) * D + (size_t)(x)]
  float c00 = mixf(T(x0, y0, z0), T(x1, y0, z0), ax);
  float c10 = mixf(T(x0, y1, z0), T(x1, y1, z0), ax);
  float c01 = mixf(T(x0, y0, z1), T(x1, y0, z1), ax);
  float c11 = mixf(T(x0, y1, z1), T(x1, y1, z1), ax);
#undef T
  float c0 = mixf(c00, c10, ay);
  float c1 = mixf(c01, c11, ay);
  return mixf(c0, c1, az);
}

EXPORT float oracle_sample_sdf(const float* sdf, uint32_t D, const float* bmin, const float* bmax,
                               const float* p) {
  return sampleSDF(sdf, D, V3(bmin[0], bmin[1], bmin[2]), V3(bmax[0], bmax[1], bmax[2]),
                   V3(p[0], p[1], p[2]));
}

/* ------------------------------------------------------------------------ */
/* GridPreSimPass: src/passes/simulation/gridPreSimPass.wgsl.ts:38-159      */
/* ------------------------------------------------------------------------ */

EXPORT void oracle_grid_pre_sim(const OracleConfig* cfg, const void* simUniforms,
                                const int32_t* densVel, const float* sdf, uint32_t sdfDims,
                                float* gradWind) {
  const OSimUniforms* U = (const OSimUniforms*)simUniforms;
  uint32_t G = cfg->gridDims;
  v3 gmin = xyz(U->gridData.boundsMin);
  v3 gmax = V3(U->gridData.boundsMax[0], U->gridData.boundsMax[1], U->gridData.boundsMax[2]);
  v3 smin = xyz(U->sdf.boundsMin), smax = xyz(U->sdf.boundsMax);
  v3 cell = div3s(sub3(gmax, gmin), (float)(G - 1u));
#pragma omp parallel for schedule(static)
  for (uint32_t id = 0; id < G * G * G; id++) {
    uint32_t z = id / (G * G);
    uint32_t idXY = id - z * G * G;
    uint32_t y = idXY / G, x = idXY % G;
    v3 pos = add3(gmin, mul3(cell, V3((float)x, (float)y, (float)z)));
    /* getWindStrength, gridPreSimPass.wgsl.ts:89-108 */
    float wind;
    float d = sampleSDF(sdf, sdfDims, smin, smax, pos);
    if (d < 0.0f) wind = 0.0f;
    else {
      v3 nd = norm3(xyz(U->wind));
      v3 toward = V3(-nd.x, -nd.y, -nd.z);
      v3 rp = add3(pos, mul3s(mul3s(toward, d), U->windColisionTraceOffset));
      float d2 = sampleSDF(sdf, sdfDims, smin, smax, rp);
      wind = d2 < 0.0f ? 0.5f : 1.0f;
    }
    /* getDensityGradient, gridPreSimPass.wgsl.ts:111-159 */
    uint32_t idx0 = gridIdx(G, x, y, z);
    float d0 = gridDecode(densVel[4u * idx0 + 3u]);
    v3 g = V3(0, 0, 0);
    static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    for (int k = 0; k < 6; k++) {
      int64_t ox = (int64_t)x + off[k][0], oy = (int64_t)y + off[k][1], oz = (int64_t)z + off[k][2];
      v3 r = V3(0, 0, 0);
      if (!(ox < 0 || oy < 0 || oz < 0)) {
        uint32_t idxO = gridIdx(G, (uint32_t)ox, (uint32_t)oy, (uint32_t)oz);
        if (idxO != idx0) {
          float dO = gridDecode(densVel[4u * idxO + 3u]);
          float diff = d0 - dO;
          r = mul3s(V3((float)off[k][0], (float)off[k][1], (float)off[k][2]), fmax_(diff, 0.0f));
        }
      }
      g = add3(g, r);
    }
    float* o = gradWind + 4u * idx0;
    o[0] = g.x; o[1] = g.y; o[2] = g.z; o[3] = wind;
  }
}

/* ------------------------------------------------------------------------ */
/* HairSimIntegrationPass: hairSimIntegrationPass.wgsl.ts:79-273 with       */
/* shaderImpl/{integration,constraints,collisions}.wgsl.ts                   */
/* ------------------------------------------------------------------------ */

/* SDF_CELL_SIZE, collisions.wgsl.ts:23-24 (a WGSL abstract-float constant) */
#define SDF_SAMPLE_GRAD_OFFSET ((float)(0.0033918858971446753 * 0.1))

/* verletIntegration, integration.wgsl.ts:8-28 */
static inline v4 verlet(float dt, v4 prev, v4 now, v3 gridDisp, float friction, v3 acc) {
  v3 pd = sub3(xyz(now), xyz(prev));
  v3 fpd = mix3(pd, gridDisp, friction);
  v3 next = add3(add3(xyz(now), fpd), mul3s(mul3s(acc, dt), dt));
  v3 r = mix3(xyz(prev), next, now.w);
  return V4(r.x, r.y, r.z, now.w);
}

static inline void add4xyz(v4* p, v3 d) { p->x = p->x + d.x; p->y = p->y + d.y; p->z = p->z + d.z; }

EXPORT void oracle_sim_integrate(const OracleConfig* cfg, const void* simUniforms, const void* hairData,
                                 float* positionsPrev /* in: prev, out: next */,
                                 const float* positionsNow, const float* positionsInitial,
                                 const float* segmentLengths, const int32_t* densVel,
                                 const float* gradWind, const float* sdf, uint32_t sdfDims) {
  const OSimUniforms* U = (const OSimUniforms*)simUniforms;
  const OHairData* HD = (const OHairData*)hairData;
  uint32_t G = cfg->gridDims;
  uint32_t S = HD->strandsCount, P = HD->pointsPerStrand, segCount = P - 1u;
  float dt = U->deltaTime;
  uint32_t iters = U->constraintIterations;
  v3 gmin = xyz(U->gridData.boundsMin);
  v3 gmax = V3(U->gridData.boundsMax[0], U->gridData.boundsMax[1], U->gridData.boundsMax[2]);
  v3 smin = xyz(U->sdf.boundsMin), smax = xyz(U->sdf.boundsMax);
  float sdfOffset = U->sdf.boundsMax.w; /* getSDF_Offset */
  v3 gravityForce = V3(0.0f, -U->gravity, 0.0f);
  v4 wind = U->wind;
#pragma omp parallel
  {
  v4* wk = (v4*)malloc(sizeof(v4) * P);
#pragma omp for schedule(static)
  for (uint32_t strand = 0; strand < S; strand++) {
    const float* pn = positionsNow + 4u * (size_t)strand * P;
    const float* pp = positionsPrev + 4u * (size_t)strand * P;
    const float* pi = positionsInitial + 4u * (size_t)strand * P;
#define LD(a, i) V4((a)[4u * (i)], (a)[4u * (i) + 1u], (a)[4u * (i) + 2u], (a)[4u * (i) + 3u])
    wk[0] = LD(pn, 0u);
    for (uint32_t i = 1; i < P; i++) {
      v4 posPrev = LD(pp, i), posNow = LD(pn, i);
      v3 force = gravityForce;
      v3 grad; float windStr; v3 vel; float dens;
      gatherGradWind(G, gradWind, gmin, gmax, xyz(posNow), &grad, &windStr);
      gatherDensityVelocity(G, densVel, gmin, gmax, xyz(posNow), &vel, &dens);
      float timer = (float)U->frameIdx * 0.73f + U->windPhaseOffset * (float)strand;
      float windJitter = fractf(timer * U->windStrengthFrequency);
      float jitterDelta = mixf(-0.5f * U->windStrengthJitter, 0.5f * U->windStrengthJitter, windJitter);
      float jitterStr = 1.0f + jitterDelta;
      float windCellStr = sat(mixf(U->windStrengthLull, 1.0f, windStr));
      force = add3(force, mul3s(xyz(wind), fabsf(wind.w * jitterStr * windCellStr)));
      force = add3(force, mul3s(grad, U->volumePreservation));
      v3 gridDisp = dens > 0.0f ? div3s(vel, dens) : V3(0, 0, 0);
      wk[i] = verlet(dt, posPrev, posNow, gridDisp, U->friction, force);
    }

    for (uint32_t it = 0; it < iters; it++) {
      /* length constraint, hairSimIntegrationPass.wgsl.ts:176-190 + constraints.wgsl.ts:5-28 */
      float kLen = U->stiffnessLengthConstr;
      v4 a = wk[0];
      for (uint32_t j = 0; j < segCount; j++) {
        v4 b = wk[j + 1u];
        float expected = segmentLengths[(size_t)strand * P + j];
        float w0 = a.w, w1 = b.w;
        v3 tng = sub3(xyz(b), xyz(a));
        float actual = len3(tng);
        float corr = 1.0f - expected / actual;
        float df = corr * kLen / (w0 + w1 + FLOAT_EPSILON);
        v3 delta = mul3s(tng, df);
        add4xyz(&a, mul3s(delta, w0));
        b.x = b.x - w1 * delta.x; b.y = b.y - w1 * delta.y; b.z = b.z - w1 * delta.z;
        wk[j] = a;
        wk[j + 1u] = b;
        a = b;
      }
      /* global shape, hairSimIntegrationPass.wgsl.ts:193-206 + constraints.wgsl.ts:31-49 */
      float kGlob = U->stiffnessGlobalConstr / (float)iters;
      for (uint32_t j = 1; j < P; j++) {
        float x = (float)j / (float)(P - 1u);
        float att = 1.0f - sat((x - U->globalConstrExtent) / U->globalConstrFade);
        v4 pinit = LD(pi, j);
        float k = kGlob * att;
        v4 p = wk[j];
        v3 dv = sub3(xyz(pinit), xyz(p));
        add4xyz(&wk[j], mul3s(mul3s(dv, p.w), k));
      }
      /* local shape, hairSimIntegrationPass.wgsl.ts:209-232 + constraints.wgsl.ts:54-120 */
      float kLoc = U->stiffnessLocalConstr / (float)iters;
      uint32_t jj = 0;
      for (; jj < P - 3u; jj++) {
        v4 i0 = LD(pi, jj), i1 = LD(pi, jj + 1u), i2 = LD(pi, jj + 2u);
        v3 cI = div3s(add3(add3(xyz(i0), xyz(i1)), xyz(i2)), 3.0f);
        float h0 = len3(sub3(cI, xyz(i1)));
        v4 p0 = wk[jj], p1 = wk[jj + 1u], p2 = wk[jj + 2u];
        v3 c = div3s(add3(add3(xyz(p0), xyz(p1)), xyz(p2)), 3.0f);
        v3 hv = sub3(xyz(p1), c);
        float h = len3(hv);
        float wT = (i0.w + 2.0f * i1.w) + i2.w;
        float w0 = i0.w / wT * 2.0f;
        float w1 = i1.w / wT * -4.0f;
        float w2 = i2.w / wT * 2.0f;
        v3 delta = mul3s(hv, 1.0f - h0 / h);
        add4xyz(&wk[jj], mul3s(delta, kLoc * w0));
        add4xyz(&wk[jj + 1u], mul3s(delta, kLoc * w1));
        add4xyz(&wk[jj + 2u], mul3s(delta, kLoc * w2));
      }
      for (; jj < P; jj++) {
        v4 i0 = LD(pi, jj - 1u), i1 = LD(pi, jj);
        v3 tInit = sub3(xyz(i1), xyz(i0));
        v4 p0 = wk[jj - 1u], p1 = wk[jj];
        v3 proj = add3(xyz(p0), tInit);
        v3 delta = sub3(proj, xyz(p1));
        add4xyz(&wk[jj], mul3s(delta, kLoc * p1.w));
      }
      /* collisions, hairSimIntegrationPass.wgsl.ts:236-261 + collisions.wgsl.ts:4-61 */
      float kColl = U->stiffnessCollisions / (float)iters;
      float kSdf = U->stiffnessSDF / (float)iters;
      v4 sph = U->collisionSphere;
      for (uint32_t j = 1; j < P; j++) {
        v4 pos = wk[j];
        {
          v3 v = sub3(xyz(pos), xyz(sph));
          float dist = len3(v) - sph.w;
          float dts = fmax_(0.0f, -dist);
          add4xyz(&pos, mul3s(mul3s(norm3(v), dts), kColl));
        }
        if (j > 2u) {
          v3 p = xyz(pos);
          float d = sampleSDF(sdf, sdfDims, smin, smax, p);
          float dOff = d + sdfOffset;
          if (!(dOff >= 0.0f)) {
            v3 cd;
            const float o = SDF_SAMPLE_GRAD_OFFSET;
            cd.x = sampleSDF(sdf, sdfDims, smin, smax, add3(p, V3(o * 1.0f, o * 0.0f, o * 0.0f)));
            cd.y = sampleSDF(sdf, sdfDims, smin, smax, add3(p, V3(o * 0.0f, o * 1.0f, o * 0.0f)));
            cd.z = sampleSDF(sdf, sdfDims, smin, smax, add3(p, V3(o * 0.0f, o * 0.0f, o * 1.0f)));
            cd = sub3(cd, V3(d, d, d));
            v3 corr = mul3s(norm3(cd), -dOff);
            add4xyz(&pos, mul3s(corr, kSdf));
          }
        }
        wk[j] = pos;
      }
    }
    float* out = positionsPrev + 4u * (size_t)strand * P;
    for (uint32_t i = 0; i < P; i++) {
      out[4u * i] = wk[i].x; out[4u * i + 1u] = wk[i].y; out[4u * i + 2u] = wk[i].z; out[4u * i + 3u] = wk[i].w;
    }
#undef LD
  }
  free(wk);
  }
}

/* ------------------------------------------------------------------------ */
/* GridPostSimPass: gridPostSimPass.wgsl.ts:45-72 and                       */
/* _addGridDensityVelocity, densityVelocityGrid.wgsl.ts:93-124              */
/* ------------------------------------------------------------------------ */

/* densVel must be zeroed by the caller (clearDensityVelocityBuffer). The
 * integer adds wrap (two's complement), like WGSL atomicAdd<i32>. */
EXPORT void oracle_grid_post_sim(const OracleConfig* cfg, const void* simUniforms, const void* hairData,
                                 const float* positionsPrev, const float* positionsNow, int32_t* densVel) {
  const OSimUniforms* U = (const OSimUniforms*)simUniforms;
  const OHairData* HD = (const OHairData*)hairData;
  uint32_t G = cfg->gridDims;
  v3 gmin = xyz(U->gridData.boundsMin);
  v3 gmax = V3(U->gridData.boundsMax[0], U->gridData.boundsMax[1], U->gridData.boundsMax[2]);
  uint32_t N = HD->strandsCount * HD->pointsPerStrand;
  uint32_t* g = (uint32_t*)densVel;
#pragma omp parallel for schedule(static)
  for (uint32_t i = 0; i < N; i++) {
    v3 pp = V3(positionsPrev[4u * i], positionsPrev[4u * i + 1u], positionsPrev[4u * i + 2u]);
    v3 pn = V3(positionsNow[4u * i], positionsNow[4u * i + 1u], positionsNow[4u * i + 2u]);
    v3 vel = sub3(pn, pp);
    GridCo co = getGridCell(G, gmin, gmax, pn);
    for (uint32_t z = co.mn[2]; z <= co.mx[2]; z++)
      for (uint32_t y = co.mn[1]; y <= co.mx[1]; y++)
        for (uint32_t x = co.mn[0]; x <= co.mx[0]; x++) {
          uint32_t idx = gridIdx(G, x, y, z);
          v3 w = cellWeights(x, y, z, co.pInGrid);
          v3 cv = mul3(vel, w);
#pragma omp atomic
          g[4u * idx + 0u] += (uint32_t)gridEncode(cv.x);
#pragma omp atomic
          g[4u * idx + 1u] += (uint32_t)gridEncode(cv.y);
#pragma omp atomic
          g[4u * idx + 2u] += (uint32_t)gridEncode(cv.z);
#pragma omp atomic
          g[4u * idx + 3u] += (uint32_t)gridEncode(len3(w));
        }
  }
}

/* ------------------------------------------------------------------------ */
/* HairShadingPass: src/passes/hairShadingPass/hairShadingPass.wgsl.ts:61-282 */
/* and marschner.wgsl.ts:19-170; shadows sampleShadows.wgsl.ts:21-150;      */
/* AO textureAo.wgsl.ts:7-12; linearizeDepth linearDepth.wgsl.ts:9-22       */
/* ------------------------------------------------------------------------ */

typedef struct { v3 baseColor; float specular, weightTT, weightTRT, shift, roughness; } MParams;

#define SQRT_TWO_PI ((float)2.5066282746310002)
#define HAIR_F0 ((float)((1.0 - 1.55) * (1.0 - 1.55) / ((1.0 + 1.55) * (1.0 + 1.55))))

static inline float cosOfHalfAngle(float c) { return sqrtf(sat(0.5f + 0.5f * c)); }

static inline float longitudinalGaussian(float si, float sr, float alpha, float beta) {
  float a = si + sr - alpha;
  float b = -(a * a) / (2.0f * beta * beta);
  return expf(b) / (beta * SQRT_TWO_PI);
}

static inline v3 pow3s(v3 b, float e) { return V3(powf(b.x, e), powf(b.y, e), powf(b.z, e)); }

static v3 hairSpecularMarschner(const MParams* p, v3 toLight, v3 toCamera, v3 tangent) {
  float sin_i = dot3(tangent, toLight);
  float sin_r = dot3(tangent, toCamera);
  float cos_i = sqrtf(fmax_(0.0f, 1.0f - sin_i * sin_i));
  float cos_r = sqrtf(fmax_(0.0f, 1.0f - sin_r * sin_r));
  float cos_d_full = cos_i * cos_r + sin_i * sin_r;
  float cos_d = cosOfHalfAngle(cos_d_full);
  v3 lightPerp = sub3(toLight, mul3s(tangent, sin_i));
  v3 cameraPerp = sub3(toCamera, mul3s(tangent, sin_r));
  float cos_phi = dot3(lightPerp, cameraPerp) * (1.0f / sqrtf(len3(lightPerp) * len3(cameraPerp) + 1e-4f));
  float cos_half_phi = cosOfHalfAngle(cos_phi);
  /* R */
  float alpha = -2.0f * p->shift;
  float beta = p->roughness * p->roughness;
  float M_r = longitudinalGaussian(sin_i, sin_r, alpha, beta);
  float N_r = 0.25f * cos_half_phi * FresnelSchlick1(cos_d, HAIR_F0);
  /* TT */
  alpha = p->shift;
  beta = 0.5f * p->roughness * p->roughness;
  float M_tt = longitudinalGaussian(sin_i, sin_r, alpha, beta);
  v3 N_tt;
  {
    float eta_prime = (1.19f / cos_d) + (0.36f * cos_d);
    float a = 1.0f / eta_prime;
    float h = (1.0f + a * (0.6f - 0.8f * cos_phi)) * cos_half_phi;
    float num = sqrtf(1.0f - h * h * a * a);
    float den = 2.0f * cos_d;
    v3 T = pow3s(p->baseColor, num / den);
    float D = expf(-3.65f * cos_phi - 3.98f);
    float fa = cos_d * sqrtf(sat(1.0f - h * h));
    float f = FresnelSchlick1(fa, HAIR_F0);
    float fTT = (1.0f - f) * (1.0f - f);
    N_tt = mul3s(mul3s(T, fTT), D);
  }
  /* TRT */
  alpha = 4.0f * p->shift;
  beta = 2.0f * p->roughness * p->roughness;
  float M_trt = longitudinalGaussian(sin_i, sin_r, alpha, beta);
  v3 N_trt;
  {
    v3 T = pow3s(p->baseColor, 0.8f / cos_d);
    float D = expf(17.0f * cos_phi - 16.78f);
    float fa = cos_d * 0.5f;
    float f = FresnelSchlick1(fa, HAIR_F0);
    float fTRT = (1.0f - f) * (1.0f - f) * f;
    N_trt = mul3s(mul3s(T, fTRT), D);
  }
  float r = p->specular * M_r * N_r;
  v3 tt = mul3s(N_tt, p->weightTT * M_tt);
  v3 trt = mul3s(N_trt, p->weightTRT * M_trt);
  return add3(add3(V3(r, r, r), tt), trt);
}

/* hairShading, hairShadingPass.wgsl.ts:166-205 */
static v3 hairShading(const MParams* p, const OLight* light, v3 toCamera, v3 tangentWS, v3 positionWS,
                      float shadow, float aoTerm) {
  v3 toLight = norm3(sub3(xyz(light->position), positionWS));
  /* KajiyaKayDiffuse */
  v3 diffuse = mul3s(p->baseColor, mixf(0.25f, 1.0f, dot3(tangentWS, toLight)));
  /* fakeMultipleScattering */
  v3 fakeNormal = norm3(sub3(toCamera, mul3s(tangentWS, dot3(toCamera, tangentWS))));
  float NoL = sat(dot3(fakeNormal, toLight));
  float diffuseScatter = (NoL + 1.0f) / (4.0f * PI_F);
  float luma = toLuma(p->baseColor);
  v3 tint = pow3s(div3s(p->baseColor, luma), 1.0f - shadow);
  v3 sq = V3(sqrtf(p->baseColor.x), sqrtf(p->baseColor.y), sqrtf(p->baseColor.z));
  v3 ms = mul3(mul3s(sq, diffuseScatter), tint);
  v3 diffuseTotal = mul3s(mul3(diffuse, ms), sat(dot3(tangentWS, toLight)));
  v3 spec = hairSpecularMarschner(p, toLight, toCamera, tangentWS);
  v3 brdf = add3(diffuseTotal, spec);
  v3 radiance = mul3s(mul3s(xyz(light->colorAndEnergy), 1.0f), light->colorAndEnergy.w);
  return mul3s(mul3(brdf, radiance), 1.0f - aoTerm);
}

/* textureGather with clamp-to-edge addressing (components x,y,z,w =
 * (i0,j1), (i1,j1), (i1,j0), (i0,j0)); the average of the four. */
static inline float gatherAvg(const float* sm, uint32_t n, v2 uv) {
  float u = uv.x * (float)n - 0.5f, v = uv.y * (float)n - 0.5f;
  int64_t i0 = (int64_t)floorf(u), j0 = (int64_t)floorf(v);
  float gx = loadTex2D(sm, n, n, i0, j0 + 1);
  float gy = loadTex2D(sm, n, n, i0 + 1, j0 + 1);
  float gz = loadTex2D(sm, n, n, i0 + 1, j0);
  float gw = loadTex2D(sm, n, n, i0, j0);
  return (gx + gy + gz + gw) / 4.0f;
}

/* calculateDirectionalShadow + _sampleShadowMap + _isValidShadowSample */
static float directionalShadow(const ORenderUniforms* U, const float* sm, uint32_t n, v3 posWS, v3 normalWS,
                               v3 posSS) {
  if (sm == NULL) return 0.0f; /* all-1.0 shadow map: never in shadow */
  v3 toSrc = norm3(sub3(xyz(U->shadows.sourcePosition), posWS));
  float bias = fmax_(fabsf(U->shadows.bias) * (1.0f - dot3(normalWS, toSrc)), 0.0005f);
  int32_t radius = (int32_t)U->shadows.PCF_Radius;
  if (U->shadows.usePCSS > 0u) {
    float avg = gatherAvg(sm, n, V2(posSS.x, posSS.y));
    float dd = fmax_(posSS.z - avg, 0.0f);
    radius = 1 + f2i(dd / avg * 10.0f);
  }
  float texel = 1.0f / (float)n;
  float shadow = 0.0f;
  for (int32_t x = -radius; x <= radius; x++)
    for (int32_t y = -radius; y <= radius; y++) {
      v2 off = V2((float)x * texel, (float)y * texel);
      float avg = gatherAvg(sm, n, V2(posSS.x + off.x, posSS.y + off.y));
      shadow += (posSS.z - bias > avg) ? 1.0f : 0.0f;
    }
  float pcf = (float)(radius * 2 + 1);
  float result = shadow / (pcf * pcf);
  if (posSS.z > 1.0f) return 0.0f;
  if (posSS.x < 0.0f || posSS.x > 1.0f || posSS.y < 0.0f || posSS.y > 1.0f) return 0.0f;
  return result;
}

static inline float linearizeDepth(float n, float f, float d) { return n * f / (f + (n - f) * d); }

/*
 * depth: W*H (row 0 = top); ao: aoW*aoH or NULL (= 1.0); shadowMap: smSize^2
 * or NULL (= 1.0).  shading: S*SP vec4f output.
 */
/* ---- HwHairPass's depth (hwHairPass.ts:71-160, hwRasterizeHair.wgsl.ts:23-57,
 * index order hairIndexBuffer.ts:29-46), with the rasterizer rules the CUDA
 * prepass uses: coverage at pixel centres, both windings, edges inclusive,
 * depth = NDC z interpolated with the screen-space barycentric weights,
 * (w0 z0 + w1 z1 + w2 z2) / area,
 * triangles with a vertex behind the camera not drawn, depth outside [0, 1]
 * discarded, depth test 'less' (the minimum). ---- */
typedef struct { float x, y, z; int ok; } OScreenV;

static float hdEdge(float ax, float ay, float bx, float by, float px, float py) {
  return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

static void hdQuad(const ORenderUniforms* U, const float* pos, const float* tan, uint32_t P, uint32_t strand,
                   uint32_t seg, OScreenV q[4]) {
  float W = U->viewport.x, H = U->viewport.y;
  for (uint32_t k = 0; k < 4u; k++) {
    size_t i = (size_t)strand * P + seg + (k >> 1);
    const float* p = pos + 4 * i;
    const float* t = tan + 4 * i;
    v4 pVS = m4v(&U->modelViewMat, V4(p[0], p[1], p[2], 1.0f));
    v4 tVS = m4v(&U->modelViewMat, V4(t[0], t[1], t[2], 1.0f));
    v3 c = cross3(xyz(tVS), V3(0.0f, 0.0f, 1.0f));
    v3 right = dot3(c, c) >= 1e-7f ? norm3(c) : V3(0.0f, 0.0f, 0.0f); /* safeNormalize3 */
    v3 th = mul3s(right, U->fiberRadius);
    v3 e = (k & 1u) ? sub3(xyz(pVS), th) : add3(xyz(pVS), th);
    v4 clip = m4v(&U->projMatrix, V4(e.x, e.y, e.z, 1.0f));
    OScreenV v;
    v.ok = clip.w > 0.0f;
    float nx = clip.x / clip.w, ny = clip.y / clip.w;
    v.z = clip.z / clip.w;
    v.x = (nx * 0.5f + 0.5f) * W;
    v.y = (0.5f - ny * 0.5f) * H;
    q[k] = v;
  }
}

static void hdTriangle(const OScreenV* a, const OScreenV* b, const OScreenV* c, uint32_t W, uint32_t H,
                       float* depth) {
  if (!a->ok || !b->ok || !c->ok) return;
  float area = hdEdge(a->x, a->y, b->x, b->y, c->x, c->y);
  if (!(area != 0.0f) || !isfinite(area)) return;
  float mnx = fminf(fminf(a->x, b->x), c->x), mxx = fmaxf(fmaxf(a->x, b->x), c->x);
  float mny = fminf(fminf(a->y, b->y), c->y), mxy = fmaxf(fmaxf(a->y, b->y), c->y);
  if (!(mxx >= 0.5f && mxy >= 0.5f && mnx <= (float)W - 0.5f && mny <= (float)H - 0.5f)) return;
  int x0 = (int)fmaxf(ceilf(mnx - 0.5f), 0.0f), y0 = (int)fmaxf(ceilf(mny - 0.5f), 0.0f);
  int x1 = (int)fminf(floorf(mxx - 0.5f), (float)W - 1.0f), y1 = (int)fminf(floorf(mxy - 0.5f), (float)H - 1.0f);
  float aa = fabsf(area);
  for (int y = y0; y <= y1; y++)
    for (int x = x0; x <= x1; x++) {
      float px = (float)x + 0.5f, py = (float)y + 0.5f;
      float w0 = hdEdge(b->x, b->y, c->x, c->y, px, py);
      float w1 = hdEdge(c->x, c->y, a->x, a->y, px, py);
      float w2 = hdEdge(a->x, a->y, b->x, b->y, px, py);
      if (area < 0.0f) { w0 = -w0; w1 = -w1; w2 = -w2; }
      if (!(w0 >= 0.0f && w1 >= 0.0f && w2 >= 0.0f)) continue;
      float z = (w0 * a->z + w1 * b->z + w2 * c->z) / aa;
      if (!(z >= 0.0f && z <= 1.0f)) continue;
      z = z + 0.0f;
      float* d = depth + (size_t)y * W + x;
      if (z < *d) *d = z;
    }
}

/* depth: W*H f32, the scene depth on entry, with the hair drawn on exit */
EXPORT void oracle_hair_depth(const void* uniforms, const void* hairData, const float* positions,
                              const float* tangents, uint32_t strandsToRender, float* depth) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  const OHairData* HD = (const OHairData*)hairData;
  uint32_t W = f2u(U->viewport.x), H = f2u(U->viewport.y);
  uint32_t P = HD->pointsPerStrand, S = HD->strandsCount;
  uint32_t nStrands = strandsToRender < S ? strandsToRender : S;
  for (uint32_t strand = 0; strand < nStrands; strand++)
    for (uint32_t seg = 0; seg + 1u < P; seg++) {
      OScreenV q[4];
      hdQuad(U, positions, tangents, P, strand, seg, q);
      hdTriangle(&q[0], &q[1], &q[2], W, H, depth);
      hdTriangle(&q[2], &q[1], &q[3], W, H, depth);
    }
}

/* HwHairPass's normal output (hwHairPass.wgsl.ts:60-97): the winning
 * fragment at each pixel is the first in draw order (strand, segment,
 * triangle) whose depth equals hairDepth; its tangent (modelMatrix *
 * (tangent, 1), interpolated with perspective-correct barycentrics: screen
 * barycentrics b_i over w_i) normalised, octahedron-encoded
 * (shaderSnippets.wgls.ts:25-46) and stored as f16 (rg16float).  normals:
 * W*H*2 floats, in/out. */
typedef struct { OScreenV s; float w; v3 t; } ONVert;

static void hnVert(const ORenderUniforms* U, const float* pos, const float* tan, size_t i, int plus, ONVert* out) {
  float W = U->viewport.x, H = U->viewport.y;
  const float* p = pos + 4 * i;
  const float* t = tan + 4 * i;
  v4 pVS = m4v(&U->modelViewMat, V4(p[0], p[1], p[2], 1.0f));
  v4 tVS = m4v(&U->modelViewMat, V4(t[0], t[1], t[2], 1.0f));
  v3 c = cross3(xyz(tVS), V3(0.0f, 0.0f, 1.0f));
  v3 right = dot3(c, c) >= 1e-7f ? norm3(c) : V3(0.0f, 0.0f, 0.0f);
  v3 th = mul3s(right, U->fiberRadius);
  v3 e = plus ? add3(xyz(pVS), th) : sub3(xyz(pVS), th);
  v4 clip = m4v(&U->projMatrix, V4(e.x, e.y, e.z, 1.0f));
  out->s.ok = clip.w > 0.0f;
  float nx = clip.x / clip.w, ny = clip.y / clip.w;
  out->s.z = clip.z / clip.w;
  out->s.x = (nx * 0.5f + 0.5f) * W;
  out->s.y = (0.5f - ny * 0.5f) * H;
  out->w = clip.w;
  out->t = xyz(m4v(&U->modelMatrix, V4(t[0], t[1], t[2], 1.0f)));
}

static void hnOct(v3 t0, float* out) {
  v3 t = norm3(t0);
  float s = (fabsf(t.x) + fabsf(t.y)) + fabsf(t.z);
  float nx = t.x / s, ny = t.y / s, nz = t.z / s;
  if (nz < 0.0f) {
    float sx = nx >= 0.0f ? 1.0f : -1.0f, sy = ny >= 0.0f ? 1.0f : -1.0f;
    float ax = (1.0f - fabsf(ny)) * sx, ay = (1.0f - fabsf(nx)) * sy;
    nx = ax;
    ny = ay;
  }
  out[0] = f16_to_f32(f32_to_f16_rne(nx * 0.5f + 0.5f));
  out[1] = f16_to_f32(f32_to_f16_rne(ny * 0.5f + 0.5f));
}

EXPORT void oracle_hair_normals(const void* uniforms, const void* hairData, const float* positions,
                                const float* tangents, uint32_t strandsToRender, const float* hairDepth,
                                float* normals) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  const OHairData* HD = (const OHairData*)hairData;
  uint32_t W = f2u(U->viewport.x), H = f2u(U->viewport.y);
  uint32_t P = HD->pointsPerStrand, S = HD->strandsCount;
  uint32_t nStrands = strandsToRender < S ? strandsToRender : S;
  uint32_t* win = (uint32_t*)malloc((size_t)W * H * 4);
  for (size_t i = 0; i < (size_t)W * H; i++) win[i] = 0xFFFFFFFFu;
  for (uint32_t strand = 0; strand < nStrands; strand++)
    for (uint32_t seg = 0; seg + 1u < P; seg++) {
      OScreenV q[4];
      hdQuad(U, positions, tangents, P, strand, seg, q);
      for (uint32_t tr = 0; tr < 2u; tr++) {
        const OScreenV* a = tr ? &q[2] : &q[0];
        const OScreenV* b = &q[1];
        const OScreenV* c = tr ? &q[3] : &q[2];
        if (!a->ok || !b->ok || !c->ok) continue;
        float area = hdEdge(a->x, a->y, b->x, b->y, c->x, c->y);
        if (!(area != 0.0f) || !isfinite(area)) continue;
        float mnx = fminf(fminf(a->x, b->x), c->x), mxx = fmaxf(fmaxf(a->x, b->x), c->x);
        float mny = fminf(fminf(a->y, b->y), c->y), mxy = fmaxf(fmaxf(a->y, b->y), c->y);
        if (!(mxx >= 0.5f && mxy >= 0.5f && mnx <= (float)W - 0.5f && mny <= (float)H - 0.5f)) continue;
        int x0 = (int)fmaxf(ceilf(mnx - 0.5f), 0.0f), y0 = (int)fmaxf(ceilf(mny - 0.5f), 0.0f);
        int x1 = (int)fminf(floorf(mxx - 0.5f), (float)W - 1.0f), y1 = (int)fminf(floorf(mxy - 0.5f), (float)H - 1.0f);
        float aa = fabsf(area);
        uint32_t prim = ((strand * (P - 1u) + seg) << 1) | tr;
        for (int y = y0; y <= y1; y++)
          for (int x = x0; x <= x1; x++) {
            float px = (float)x + 0.5f, py = (float)y + 0.5f;
            float w0 = hdEdge(b->x, b->y, c->x, c->y, px, py);
            float w1 = hdEdge(c->x, c->y, a->x, a->y, px, py);
            float w2 = hdEdge(a->x, a->y, b->x, b->y, px, py);
            if (area < 0.0f) { w0 = -w0; w1 = -w1; w2 = -w2; }
            if (!(w0 >= 0.0f && w1 >= 0.0f && w2 >= 0.0f)) continue;
            float z = (w0 * a->z + w1 * b->z + w2 * c->z) / aa;
            if (!(z >= 0.0f && z <= 1.0f)) continue;
            z = z + 0.0f;
            size_t pi = (size_t)y * W + x;
            uint32_t zb, db;
            memcpy(&zb, &z, 4);
            memcpy(&db, &hairDepth[pi], 4);
            if (zb == db && win[pi] == 0xFFFFFFFFu) win[pi] = prim;
          }
      }
    }
  for (size_t pi = 0; pi < (size_t)W * H; pi++) {
    uint32_t prim = win[pi];
    if (prim == 0xFFFFFFFFu) continue;
    uint32_t tr = prim & 1u, segIdx = prim >> 1, strand = segIdx / (P - 1u), seg = segIdx - strand * (P - 1u);
    size_t pt = (size_t)strand * P + seg;
    ONVert q[4];
    hnVert(U, positions, tangents, pt, 1, &q[0]);
    hnVert(U, positions, tangents, pt, 0, &q[1]);
    hnVert(U, positions, tangents, pt + 1u, 1, &q[2]);
    hnVert(U, positions, tangents, pt + 1u, 0, &q[3]);
    const ONVert* v0 = tr ? &q[2] : &q[0];
    const ONVert* v1 = &q[1];
    const ONVert* v2 = tr ? &q[3] : &q[2];
    float px = (float)(pi % W) + 0.5f, py = (float)(pi / W) + 0.5f;
    float area = hdEdge(v0->s.x, v0->s.y, v1->s.x, v1->s.y, v2->s.x, v2->s.y);
    float b0 = hdEdge(v1->s.x, v1->s.y, v2->s.x, v2->s.y, px, py);
    float b1 = hdEdge(v2->s.x, v2->s.y, v0->s.x, v0->s.y, px, py);
    float b2 = hdEdge(v0->s.x, v0->s.y, v1->s.x, v1->s.y, px, py);
    if (area < 0.0f) { b0 = -b0; b1 = -b1; b2 = -b2; }
    float a = fabsf(area);
    float p0 = (b0 / a) / v0->w, p1 = (b1 / a) / v1->w, p2 = (b2 / a) / v2->w;
    float sum = (p0 + p1) + p2;
    v3 t = V3(((p0 * v0->t.x + p1 * v1->t.x) + p2 * v2->t.x) / sum, ((p0 * v0->t.y + p1 * v1->t.y) + p2 * v2->t.y) / sum,
              ((p0 * v0->t.z + p1 * v1->t.z) + p2 * v2->t.z) / sum);
    hnOct(t, normals + 2 * pi);
  }
  free(win);
}

/* AoPass + GTAO (aoPass.wgsl.ts main_fs, gtao.wgsl.ts): see the CUDA pass;
 * out: ceil(W * scale) x ceil(H * scale) floats, r16float values.  Loads
 * outside the textures read 0; a negative coordinate saturates to 0. */
typedef struct { const float* depth; uint32_t W, H; float vw, vh; const mat4* pinv; } OGtao;

static float aoLoadDepth(const OGtao* a, float px, float py) {
  uint32_t x = f2u(px), y = f2u(py);
  return x < a->W && y < a->H ? a->depth[(size_t)y * a->W + x] : 0.0f;
}
static float aoLin(float d) { return (0.01f * 100.0f) / (100.0f + (0.01f - 100.0f) * d); }
static v3 aoReproject(const OGtao* a, float px, float py) {
  float d = aoLoadDepth(a, px, py);
  float x = (px / a->vw) * 2.0f - 1.0f, y = (py / a->vh) * 2.0f - 1.0f;
  v4 c = m4v(a->pinv, V4(x, y, d, 1.0f));
  return V3(c.x / c.w, c.y / c.w, aoLin(d));
}
static float aoRound(float v) { return v < 0.5f ? floorf(v) : ceilf(v); }
static float aoFalloff(float dist, float s2, float e2) { return 2.0f * sat((dist - s2) / (e2 - s2)); }
static float aoFract(float x) { return x - floorf(x); }
static v3 aoDecodeOct(float fx0, float fy0) {
  float fx = fx0 * 2.0f - 1.0f, fy = fy0 * 2.0f - 1.0f;
  v3 n = V3(fx, fy, (1.0f - fabsf(fx)) - fabsf(fy));
  float t = sat(-n.z);
  n.x = n.x >= 0.0f ? n.x - t : n.x + t;
  n.y = n.y >= 0.0f ? n.y - t : n.y + t;
  return norm3(n);
}

EXPORT void oracle_gtao(const void* uniforms, const float* depth, const float* normals, float scale, float* out) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  const float PI = 3.141592653589793f, HALF_PI = 1.5707963267948966f, ZFAR = 100.0f;
  OGtao a = {depth, f2u(U->viewport.x), f2u(U->viewport.y), U->viewport.x, U->viewport.y, &U->projMatrixInv};
  uint32_t aoW = (uint32_t)ceilf(U->viewport.x * scale), aoH = (uint32_t)ceilf(U->viewport.y * scale);
  const OGtao* A = &a;
#pragma omp parallel for schedule(static)
  for (uint32_t i = 0; i < aoW * aoH; i++) {
    float px = ((float)(i % aoW) + 0.5f) / scale, py = ((float)(i / aoW) + 0.5f) / scale;
    uint32_t nx = f2u(px), ny = f2u(py);
    float no[2] = {0.0f, 0.0f};
    if (nx < A->W && ny < A->H) memcpy(no, normals + 2 * ((size_t)ny * A->W + nx), sizeof no);
    v3 normalWS = aoDecodeOct(no[0], no[1]);
    v3 posVS = aoReproject(A, px, py);
    v3 nVS = xyz(m4v(&U->viewMatrix, V4(normalWS.x, normalWS.y, normalWS.z, 1.0f)));
    nVS.z = -nVS.z;
    v3 toCam = norm3(V3(-posVS.x, -posVS.y, -posVS.z));
    float ao = 0.0f;
    if (!(posVS.z >= 0.999f * ZFAR)) {
      float nSteps = (float)U->ao.numSteps;
      float radius = fmaxf(nSteps, U->ao.radius * (posVS.z / ZFAR));
      float stepSize = radius / nSteps;
      float rotJitter = PI * aoFract(52.9829189f * aoFract(px * 0.06711056f + py * 0.00583715f));
      float jitterMod = (px + py) * 0.25f;
      float radiusJitter = (aoFract(jitterMod) * stepSize) * 0.25f;
      for (uint32_t d = 0; d < U->ao.numDirections; d++) {
        float phi = (float)d * (PI / (float)U->ao.numDirections) + U->ao.directionOffset * PI;
        phi = phi + rotJitter;
        float step = 1.0f + 0.25f * stepSize;
        step = step + radiusJitter;
        float dx = cosf(phi), dy = sinf(phi);
        float h1 = -1.0f, h2 = -1.0f;
        for (uint32_t j = 0; j < U->ao.numSteps; j++) {
          float ox = aoRound(dx * step), oy = aoRound(dy * step);
          v3 s = aoReproject(A, px + ox, py + oy);
          v3 ws = sub3(s, posVS);
          float d2 = len3(ws);
          float c = dot3(ws, toCam) * (1.0f / sqrtf(d2));
          h1 = fmaxf(h1, c - aoFalloff(d2, U->ao.falloffStart2, U->ao.falloffEnd2));
          s = aoReproject(A, px - ox, py - oy);
          ws = sub3(s, posVS);
          d2 = len3(ws);
          c = dot3(ws, toCam) * (1.0f / sqrtf(d2));
          h2 = fmaxf(h2, c - aoFalloff(d2, U->ao.falloffStart2, U->ao.falloffEnd2));
          step = step + stepSize;
        }
        h1 = acosf(h1);
        h2 = acosf(h2);
        v3 dir = V3(dx, dy, 0.0f);
        v3 bit = norm3(cross3(dir, toCam));
        v3 tng = cross3(toCam, bit);
        v3 nxv = sub3(nVS, mul3s(bit, dot3(nVS, bit)));
        float nnx = len3(nxv);
        float nnxInv = 1.0f / (nnx + 1e-6f);
        float cosxi = dot3(nxv, tng) * nnxInv;
        float gamma = acosf(cosxi) - HALF_PI;
        float cosgamma = dot3(nxv, toCam) * nnxInv;
        float singamma2 = -2.0f * cosxi;
        h1 = gamma + fmaxf(-h1 - gamma, -HALF_PI);
        h2 = gamma + fminf(h2 - gamma, HALF_PI);
        float t1 = (h1 * singamma2 + cosgamma) - cosf(2.0f * h1 - gamma);
        float t2 = (h2 * singamma2 + cosgamma) - cosf(2.0f * h2 - gamma);
        ao = ao + (nnx * 0.25f) * (t1 + t2);
      }
      ao = ao / (float)U->ao.numDirections;
    }
    out[i] = f16_to_f32(f32_to_f16_rne(ao));
  }
}

/* HairCombinePass (hairCombinePass.wgsl.ts:51-89: fragment row y reads
 * result row H - 1 - y; blend src-alpha, one-minus-src-alpha over the scene
 * colour, hairCombinePass.ts:40-52) and PresentPass (presentPass.wgsl.ts
 * main_fs, DISPLAY_MODE_FINAL: 8x8 Bayer dither, dither.wgsl.ts:26-53;
 * exposure; ACES, aces.wgsl.ts:6-13; gamma), stored as unorm8 (round to
 * nearest even).  result: W*H vec4f (the pixels of HairRasterResult);
 * scene: W*H vec4f or NULL (black); out: W*H RGBA8, row 0 at the top. */
static const uint8_t PRESENT_BAYER[64] = {0,  32, 8,  40, 2,  34, 10, 42, 48, 16, 56, 24, 50, 18, 58, 26,
                                          12, 44, 4,  36, 14, 46, 6,  38, 60, 28, 52, 20, 62, 30, 54, 22,
                                          3,  35, 11, 43, 1,  33, 9,  41, 51, 19, 59, 27, 49, 17, 57, 25,
                                          15, 47, 7,  39, 13, 45, 5,  37, 63, 31, 55, 23, 61, 29, 53, 21};

static float presentAces(float x) {
  float num = x * (2.51f * x + 0.03f);
  float den = x * (2.43f * x + 0.59f) + 0.14f;
  return sat(num / den);
}

EXPORT void oracle_present(const void* uniforms, const float* result, const float* scene, uint8_t* out) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  uint32_t W = f2u(U->viewport.x), H = f2u(U->viewport.y);
  float gamma = U->colorMgmt.x, exposure = U->colorMgmt.y, ditherStr = U->colorMgmt.z;
  for (uint32_t y = 0; y < H; y++)
    for (uint32_t x = 0; x < W; x++) {
      size_t i = (size_t)y * W + x;
      const float* src = result + 4 * ((size_t)(H - 1u - y) * W + x);
      float dst[4] = {0.0f, 0.0f, 0.0f, 1.0f};
      if (scene) memcpy(dst, scene + 4 * i, sizeof dst);
      float ia = 1.0f - src[3];
      float dither = (float)PRESENT_BAYER[(y % 8u) * 8u + (x % 8u)] / 63.0f * ditherStr / 256.0f;
      for (int k = 0; k < 3; k++) {
        float v = src[k] * src[3] + dst[k] * ia;
        v = v + dither;
        v = v * exposure;
        v = presentAces(v);
        v = powf(v, 1.0f / gamma);
        out[4 * i + k] = (uint8_t)nearbyintf(sat(v) * 255.0f);
      }
      out[4 * i + 3] = 255;
    }
}

EXPORT void oracle_shading(const OracleConfig* cfg, const void* uniforms, const void* hairData,
                           const float* positions, const float* tangents, const float* depth,
                           const float* ao, uint32_t aoW, uint32_t aoH,
                           const float* shadowMap, uint32_t smSize, float* shading) {
  const ORenderUniforms* U = (const ORenderUniforms*)uniforms;
  const OHairData* HD = (const OHairData*)hairData;
  uint32_t SP = cfg->shadingPoints, P = HD->pointsPerStrand;
  v2 vp = V2(U->viewport.x, U->viewport.y);
  uint32_t W = f2u(vp.x), H = f2u(vp.y);
  const OHairMaterial* m = &U->hairMaterial;
#pragma omp parallel for schedule(static)
  for (uint32_t strand = 0; strand < HD->strandsCount; strand++) {
    for (uint32_t sp = 0; sp < SP; sp++) {
      float t = (float)sp / (float)SP;
      uint32_t i0, i1;
      float ts = remapToIndices(P, t, &i0, &i1);
      const float* a = positions + 4u * ((size_t)strand * P + i0);
      const float* b = positions + 4u * ((size_t)strand * P + i1);
      const float* tg = tangents + 4u * ((size_t)strand * P + i1);
      v3 s0 = V3(a[0], a[1], a[2]), s1 = V3(b[0], b[1], b[2]);
      v3 t0 = norm3(sub3(s1, s0));
      v3 t1 = V3(tg[0], tg[1], tg[2]);
      v3 posO = mix3(s0, s1, ts);
      v3 tanO = mix3(t0, t1, ts);
      v4 posWS = m4v(&U->modelMatrix, V4(posO.x, posO.y, posO.z, 1.0f));
      v4 tanWS = m4v(&U->modelMatrix, V4(tanO.x, tanO.y, tanO.z, 1.0f));
      v3 proj = projectVertex(&U->vpMatrix, posWS);
      v2 p01 = V2(proj.x * 0.5f + 0.5f, proj.y * 0.5f + 0.5f);
      v2 texPx = V2(vp.x * p01.x, vp.y * (1.0f - p01.y));

      v3 base = mix3(V3(m->color0[0], m->color0[1], m->color0[2]), V3(m->color1[0], m->color1[1], m->color1[2]), t);
      v3 rnd = randomRGB(strand, 1.0f);
      base = mix3(base, rnd, m->colorRng);
      float rngB = fractf((float)strand / 255.0f);
      base = mix3(base, mul3s(base, rngB), m->lumaRng);
      v3 toCam = norm3(sub3(xyz(U->cameraPosition), xyz(posWS)));
      MParams mp = {base, m->specular, m->weightTT, m->weightTRT, m->shift, m->roughness};

      /* getShadow */
      v4 pl = m4v(&U->shadows.sourceMVP_Matrix, posWS);
      v3 posSS = V3(pl.x * 0.5f + 0.5f, 1.0f - (pl.y * 0.5f + 0.5f), pl.z);
      float shadow = 1.0f - directionalShadow(U, shadowMap, smSize, xyz(posWS), xyz(tanWS), posSS);
      shadow = clampf_(shadow, 1.0f - m->shadows, 1.0f);

      /* sampleAo */
      float aov = 1.0f;
      if (ao) {
        v2 tt = V2(texPx.x / vp.x, texPx.y / vp.y);
        int32_t ax = f2i((float)aoW * tt.x), ay = f2i((float)aoH * tt.y);
        aov = loadTex2D(ao, aoW, aoH, ax, ay);
      }
      float aoT = 1.0f - mixf(1.0f, aov, U->ao.strength);

      /* getAttenuation */
      float myDepth = linearizeDepth(cfg->cameraNear, cfg->cameraFar, proj.z);
      float zb = loadTex2D(depth, W, H, (int64_t)f2u(texPx.x), (int64_t)f2u(texPx.y));
      float zbd = linearizeDepth(cfg->cameraNear, cfg->cameraFar, zb);
      float att = fabsf(myDepth - zbd) * m->attenuation;
      aoT = sat(aoT + att);

      v3 sum = V3(0, 0, 0);
      sum = add3(sum, hairShading(&mp, &U->light0, toCam, xyz(tanWS), xyz(posWS), shadow, aoT));
      sum = add3(sum, hairShading(&mp, &U->light1, toCam, xyz(tanWS), xyz(posWS), shadow, aoT));
      sum = add3(sum, hairShading(&mp, &U->light2, toCam, xyz(tanWS), xyz(posWS), shadow, aoT));
      float alpha = sp >= SP - 1u ? 0.0f : 1.0f;
      /* _setShadingPoint, hairShadingBuffer.ts:12-16 */
      float* o = shading + 4u * ((size_t)strand * SP + clampu(sp, 0u, SP - 1u));
      o[0] = sum.x; o[1] = sum.y; o[2] = sum.z; o[3] = alpha;
    }
  }
}
