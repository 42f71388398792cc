// HairShadingPass: strand-space shading, one thread per (strand, shading point).
//
// Reference WGSL: src/passes/hairShadingPass/hairShadingPass.wgsl.ts:61-282,
// marschner.wgsl.ts:19-170, shadow sampling
// src/passes/shadowMapPass/shared/sampleShadows.wgsl.ts:21-150, AO lookup
// src/passes/aoPass/shared/textureAo.wgsl.ts:7-12, linearizeDepth
// src/passes/_shaderSnippets/linearDepth.wgsl.ts:9-22.
#define HFB_TU 2
#include "hfb_internal.cuh"
#include "hfb_math.cuh"

namespace hfb {
namespace {

constexpr float PI_F = 3.141592653589793f;
constexpr float SQRT_TWO_PI = (float)2.5066282746310002;
constexpr float HAIR_F0 = (float)((1.0 - 1.55) * (1.0 - 1.55) / ((1.0 + 1.55) * (1.0 + 1.55)));

struct MParams {
  f3 baseColor;
  float specular, weightTT, weightTRT, shift, roughness;
};

__device__ __forceinline__ float FresnelSchlick1(float c, float F0) {
  return fadd(F0, fmul(fsub(1.0f, F0), powf(fsub(1.0f, c), 5.0f)));
}
__device__ __forceinline__ float cosOfHalfAngle(float c) { return sqrtf(sat(fadd(0.5f, fmul(0.5f, c)))); }
__device__ __forceinline__ float longitudinalGaussian(float si, float sr, float alpha, float beta) {
  float a = fsub(fadd(si, sr), alpha);
  float b = -fmul(a, a) / fmul(fmul(2.0f, beta), beta);
  return expf(b) / fmul(beta, SQRT_TWO_PI);
}
__device__ __forceinline__ f3 pow3s(f3 b, float e) { return {powf(b.x, e), powf(b.y, e), powf(b.z, e)}; }

// hairSpecularMarschner, marschner.wgsl.ts:34-97
__device__ f3 marschner(const MParams& p, f3 toLight, f3 toCamera, f3 tangent) {
  float sin_i = dot3(tangent, toLight);
  float sin_r = dot3(tangent, toCamera);
  float cos_i = sqrtf(fmaxf(0.0f, fsub(1.0f, fmul(sin_i, sin_i))));
  float cos_r = sqrtf(fmaxf(0.0f, fsub(1.0f, fmul(sin_r, sin_r))));
  float cos_d = cosOfHalfAngle(fadd(fmul(cos_i, cos_r), fmul(sin_i, sin_r)));
  f3 lightPerp = sub3(toLight, mul3s(tangent, sin_i));
  f3 cameraPerp = sub3(toCamera, mul3s(tangent, sin_r));
  float cos_phi = fmul(dot3(lightPerp, cameraPerp),
                       1.0f / sqrtf(fadd(fmul(len3(lightPerp), len3(cameraPerp)), 1e-4f)));
  float cos_half_phi = cosOfHalfAngle(cos_phi);
  float r2 = fmul(p.roughness, p.roughness);
  // R
  float M_r = longitudinalGaussian(sin_i, sin_r, fmul(-2.0f, p.shift), r2);
  float N_r = fmul(fmul(0.25f, cos_half_phi), FresnelSchlick1(cos_d, HAIR_F0));
  // TT
  float M_tt = longitudinalGaussian(sin_i, sin_r, p.shift, fmul(fmul(0.5f, p.roughness), p.roughness));
  f3 N_tt;
  {
    float eta = fadd(1.19f / cos_d, fmul(0.36f, cos_d));
    float a = 1.0f / eta;
    float h = fmul(fadd(1.0f, fmul(a, fsub(0.6f, fmul(0.8f, cos_phi)))), cos_half_phi);
    float num = sqrtf(fsub(1.0f, fmul(fmul(fmul(h, h), a), a)));
    float den = fmul(2.0f, cos_d);
    f3 T = pow3s(p.baseColor, num / den);
    float Dd = expf(fsub(fmul(-3.65f, cos_phi), 3.98f));
    float fa = fmul(cos_d, sqrtf(sat(fsub(1.0f, fmul(h, h)))));
    float f = FresnelSchlick1(fa, HAIR_F0);
    float fTT = fmul(fsub(1.0f, f), fsub(1.0f, f));
    N_tt = mul3s(mul3s(T, fTT), Dd);
  }
  // TRT
  float M_trt = longitudinalGaussian(sin_i, sin_r, fmul(4.0f, p.shift), fmul(fmul(2.0f, p.roughness), p.roughness));
  f3 N_trt;
  {
    f3 T = pow3s(p.baseColor, 0.8f / cos_d);
    float Dd = expf(fsub(fmul(17.0f, cos_phi), 16.78f));
    float f = FresnelSchlick1(fmul(cos_d, 0.5f), HAIR_F0);
    float fTRT = fmul(fmul(fsub(1.0f, f), fsub(1.0f, f)), f);
    N_trt = mul3s(mul3s(T, fTRT), Dd);
  }
  float r = fmul(fmul(p.specular, M_r), N_r);
  f3 tt = mul3s(N_tt, fmul(p.weightTT, M_tt));
  f3 trt = mul3s(N_trt, fmul(p.weightTRT, M_trt));
  return add3(add3(mk3(r, r, r), tt), trt);
}

// hairShading, hairShadingPass.wgsl.ts:166-205
__device__ f3 hairShading(const MParams& p, f4 lightPos, f4 lightCol, f3 toCamera, f3 tangentWS, f3 posWS,
                          float shadow, float aoTerm) {
  f3 toLight = norm3(sub3(xyz(lightPos), posWS));
  f3 diffuse = mul3s(p.baseColor, mixf(0.25f, 1.0f, dot3(tangentWS, toLight)));  // KajiyaKayDiffuse
  f3 fakeNormal = norm3(sub3(toCamera, mul3s(tangentWS, dot3(toCamera, tangentWS))));
  float NoL = sat(dot3(fakeNormal, toLight));
  float diffuseScatter = fadd(NoL, 1.0f) / fmul(4.0f, PI_F);
  float luma = dot3(mk3(0.2126729f, 0.7151522f, 0.0721750f), p.baseColor);
  f3 tint = pow3s(div3s(p.baseColor, luma), fsub(1.0f, shadow));
  f3 sq = mk3(sqrtf(p.baseColor.x), sqrtf(p.baseColor.y), sqrtf(p.baseColor.z));
  f3 ms = mul3(mul3s(sq, diffuseScatter), tint);
  f3 diffuseTotal = mul3s(mul3(diffuse, ms), sat(dot3(tangentWS, toLight)));
  f3 brdf = add3(diffuseTotal, marschner(p, toLight, toCamera, tangentWS));
  f3 radiance = mul3s(mul3s(xyz(lightCol), 1.0f), lightCol.w);
  return mul3s(mul3(brdf, radiance), fsub(1.0f, aoTerm));
}

__device__ __forceinline__ float gatherAvg(const float* sm, uint32_t n, float ux, float uy) {
  float u = fsub(fmul(ux, (float)n), 0.5f), v = fsub(fmul(uy, (float)n), 0.5f);
  int i0 = (int)floorf(u), j0 = (int)floorf(v);
  float gx = loadTex2DClamp(sm, n, n, i0, j0 + 1);
  float gy = loadTex2DClamp(sm, n, n, i0 + 1, j0 + 1);
  float gz = loadTex2DClamp(sm, n, n, i0 + 1, j0);
  float gw = loadTex2DClamp(sm, n, n, i0, j0);
  return fadd(fadd(fadd(gx, gy), gz), gw) / 4.0f;
}

// calculateDirectionalShadow + _sampleShadowMap + _isValidShadowSample,
// sampleShadows.wgsl.ts:47-150. A NULL map is the all-1.0 map: never in shadow.
__device__ float directionalShadow(const HfbUniforms& U, const float* sm, uint32_t n, f3 posWS, f3 normalWS,
                                   f3 posSS) {
  if (sm == nullptr) return 0.0f;
  f3 toSrc = norm3(sub3(mk3(U.shadows.sourcePosition.x, U.shadows.sourcePosition.y, U.shadows.sourcePosition.z),
                        posWS));
  float bias = fmaxf(fmul(fabsf(U.shadows.bias), fsub(1.0f, dot3(normalWS, toSrc))), 0.0005f);
  int radius = (int)U.shadows.PCF_Radius;
  if (U.shadows.usePCSS > 0u) {
    float avg = gatherAvg(sm, n, posSS.x, posSS.y);
    float dd = fmaxf(fsub(posSS.z, avg), 0.0f);
    radius = 1 + f2i(fmul(dd / avg, 10.0f));
  }
  float texel = 1.0f / (float)n;
  float shadow = 0.0f;
  for (int x = -radius; x <= radius; x++)
    for (int y = -radius; y <= radius; y++) {
      float avg = gatherAvg(sm, n, fadd(posSS.x, fmul((float)x, texel)), fadd(posSS.y, fmul((float)y, texel)));
      shadow = fadd(shadow, fsub(posSS.z, bias) > avg ? 1.0f : 0.0f);
    }
  float pcf = (float)(radius * 2 + 1);
  float result = shadow / fmul(pcf, pcf);
  if (posSS.z > 1.0f) return 0.0f;
  if (posSS.x < 0.0f || posSS.x > 1.0f || posSS.y < 0.0f || posSS.y > 1.0f) return 0.0f;
  return result;
}

__device__ __forceinline__ float linearizeDepth(float n, float f, float d) {
  return fmul(n, f) / fadd(f, fmul(fsub(n, f), d));
}

__device__ __forceinline__ void shadingBody(const HfbUniforms& U, uint32_t S, uint32_t P, uint32_t SP, float zNear,
                                            float zFar, const float4* __restrict__ pos,
                                            const float4* __restrict__ tan, const float* __restrict__ depth,
                                            const float* __restrict__ ao, uint32_t aoW, uint32_t aoH,
                                            const float* __restrict__ sm, uint32_t smSize,
                                            float4* __restrict__ shading, uint32_t gid) {
  if (gid >= S * SP) return;
  uint32_t strand = gid / SP, sp = gid - strand * SP;
  f2 vp = mk2(U.viewport.x, U.viewport.y);
  uint32_t W = f2u(vp.x), H = f2u(vp.y);
  const auto& m = U.hairMaterial;

  float t = (float)sp / (float)SP;
  uint32_t i0, i1;
  float ts = remapToIndices(P, t, i0, i1);
  float4 a = __ldg(HFB_G(&pos[(size_t)strand * P + i0]));
  float4 b = __ldg(HFB_G(&pos[(size_t)strand * P + i1]));
  float4 tg = __ldg(HFB_G(&tan[(size_t)strand * P + i1]));
  f3 s0 = mk3(a.x, a.y, a.z), s1 = mk3(b.x, b.y, b.z);
  f3 t0 = norm3(sub3(s1, s0));
  f3 posO = mix3(s0, s1, ts);
  f3 tanO = mix3(t0, mk3(tg.x, tg.y, tg.z), ts);
  f4 posWS = m4v(U.modelMatrix.m, mk4(posO.x, posO.y, posO.z, 1.0f));
  f4 tanWS = m4v(U.modelMatrix.m, mk4(tanO.x, tanO.y, tanO.z, 1.0f));
  f3 proj = projectVertex(U.vpMatrix.m, posWS);
  f2 p01 = mk2(fadd(fmul(proj.x, 0.5f), 0.5f), fadd(fmul(proj.y, 0.5f), 0.5f));
  f2 texPx = mk2(fmul(vp.x, p01.x), fmul(vp.y, fsub(1.0f, p01.y)));

  f3 base = mix3(mk3(m.color0[0], m.color0[1], m.color0[2]), mk3(m.color1[0], m.color1[1], m.color1[2]), t);
  float fs = (float)strand;
  f3 rnd = sat3(mk3(fractf(fmul(fs, 1.73f)), fractf(fmul(fs, 1.17f)), fractf(fmul(fs, 1.31f))));  // randomRGB(s, 1.0)
  base = mix3(base, rnd, m.colorRng);
  float rngB = fractf(fs / 255.0f);
  base = mix3(base, mul3s(base, rngB), m.lumaRng);
  f3 camPos = mk3(U.cameraPosition.x, U.cameraPosition.y, U.cameraPosition.z);
  f3 toCam = norm3(sub3(camPos, xyz(posWS)));
  MParams mp{base, m.specular, m.weightTT, m.weightTRT, m.shift, m.roughness};

  // getShadow
  f4 pl = m4v(U.shadows.sourceMVP_Matrix.m, posWS);
  f3 posSS = mk3(fadd(fmul(pl.x, 0.5f), 0.5f), fsub(1.0f, fadd(fmul(pl.y, 0.5f), 0.5f)), pl.z);
  float shadow = fsub(1.0f, directionalShadow(U, sm, smSize, xyz(posWS), xyz(tanWS), posSS));
  shadow = clampf(shadow, fsub(1.0f, m.shadows), 1.0f);

  // sampleAo
  float aov = 1.0f;
  if (ao) {
    int ax = f2i(fmul((float)aoW, texPx.x / vp.x)), ay = f2i(fmul((float)aoH, texPx.y / vp.y));
    aov = loadTex2DClamp(ao, aoW, aoH, ax, ay);
  }
  float aoT = fsub(1.0f, mixf(1.0f, aov, U.ao.strength));

  // getAttenuation
  float myDepth = linearizeDepth(zNear, zFar, proj.z);
  float zb = loadTex2DClamp(depth, W, H, (int)min(f2u(texPx.x), 0x7fffffffu), (int)min(f2u(texPx.y), 0x7fffffffu));
  float att = fmul(fabsf(fsub(myDepth, linearizeDepth(zNear, zFar, zb))), m.attenuation);
  aoT = sat(fadd(aoT, att));

  f3 sum = mk3(0.f, 0.f, 0.f);
  sum = add3(sum, hairShading(mp, ld4(make_float4(U.light0.position.x, U.light0.position.y, U.light0.position.z, U.light0.position.w)),
                              ld4(make_float4(U.light0.colorAndEnergy.x, U.light0.colorAndEnergy.y, U.light0.colorAndEnergy.z, U.light0.colorAndEnergy.w)),
                              toCam, xyz(tanWS), xyz(posWS), shadow, aoT));
  sum = add3(sum, hairShading(mp, ld4(make_float4(U.light1.position.x, U.light1.position.y, U.light1.position.z, U.light1.position.w)),
                              ld4(make_float4(U.light1.colorAndEnergy.x, U.light1.colorAndEnergy.y, U.light1.colorAndEnergy.z, U.light1.colorAndEnergy.w)),
                              toCam, xyz(tanWS), xyz(posWS), shadow, aoT));
  sum = add3(sum, hairShading(mp, ld4(make_float4(U.light2.position.x, U.light2.position.y, U.light2.position.z, U.light2.position.w)),
                              ld4(make_float4(U.light2.colorAndEnergy.x, U.light2.colorAndEnergy.y, U.light2.colorAndEnergy.z, U.light2.colorAndEnergy.w)),
                              toCam, xyz(tanWS), xyz(posWS), shadow, aoT));
  float alpha = sp >= SP - 1u ? 0.0f : 1.0f;
  *HFB_G(&shading[gid]) = make_float4(sum.x, sum.y, sum.z, alpha);  // _setShadingPoint
}

__global__ void __launch_bounds__(128)
shadingKernel(const HfbUniforms U, uint32_t S, uint32_t P, uint32_t SP, float zNear, float zFar,
              const float4* __restrict__ pos, const float4* __restrict__ tan, const float* __restrict__ depth,
              const float* __restrict__ ao, uint32_t aoW, uint32_t aoH, const float* __restrict__ sm,
              uint32_t smSize, float4* __restrict__ shading) {
  shadingBody(U, S, P, SP, zNear, zFar, pos, tan, depth, ao, aoW, aoH, sm, smSize, shading,
              blockIdx.x * blockDim.x + threadIdx.x);
}

// batched: persistent over the virtual blocks of every instance
__global__ void __launch_bounds__(128, 6) shadingBatch(BatchView b, uint32_t SP, float zNear, float zFar) {
  const uint32_t n = b.hdr->n;
  const uint32_t* row = b.prefix + BK_SHADING * (BATCH_MAX + 1);
  const uint32_t total = row[n];
  __shared__ uint32_t vbNext[2];
  uint32_t vbPar = 0;
  for (uint32_t v = batchNext(b.hdr, BK_SHADING, vbNext, vbPar); v < total; v = batchNext(b.hdr, BK_SHADING, vbNext, vbPar)) {
    const uint32_t i = batchFind(row, n, v);
    const BatchInst& I = b.insts[i];
    shadingBody(I.U, I.S, I.P, SP, zNear, zFar, I.posNew, I.tan, I.shadingDepth, I.ao, I.aoW, I.aoH, I.sm,
                I.smSize, I.shading, (v - row[i]) * 128u + threadIdx.x);
  }
}

}  // namespace

cudaError_t launchShading(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                          const float* tan, const float* depth, const float* ao, uint32_t aoW, uint32_t aoH,
                          const float* sm, uint32_t smSize, float* shading) {
  HFB_CHECK_BIND(c);
  uint32_t SP = c->cfg.shadingPoints;
  uint32_t n = h.strandsCount * SP;
  shadingKernel<<<divCeil(n, 128), 128, 0, c->stream>>>(u, h.strandsCount, h.pointsPerStrand, SP,
                                                          c->cfg.cameraNear, c->cfg.cameraFar,
                                                          (const float4*)pos, (const float4*)tan, depth, ao,
                                                          aoW, aoH, sm, smSize, (float4*)shading);
  HFB_AFTER_LAUNCH(c, "shadingKernel");
  c->launches += 1;
  return cudaGetLastError();
}

}  // namespace hfb

namespace hfb {
cudaError_t launchBatchShading(HfbCtx* c, const BatchView& b) {
  HFB_CHECK_BIND(c);
  uint32_t& grid = c->batchGrid[BK_SHADING];
  if (!grid) grid = c->smCount * 16u;
  shadingBatch<<<batchLaunchGrid(c, grid), 128, 0, c->stream>>>(b, c->cfg.shadingPoints, c->cfg.cameraNear, c->cfg.cameraFar);
  HFB_AFTER_LAUNCH(c, "shadingBatch");
  c->launches += 1;
  return cudaGetLastError();
}
}  // namespace hfb
