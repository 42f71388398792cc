// GTAO: AoPass (aoPass.wgsl.ts main_fs, gtao.wgsl.ts) as CUDA.
//
// One thread per AO texel (the AO texture is the viewport times the
// reference's textureSizeMul, 0.5): the texel's full-resolution position
// ((x + 0.5) / scale), the normal there (rg16float octahedron, decoded as
// decodeOctahedronNormal does), and gtao(): for each of numDirections
// directions, numSteps steps each way, every sample reprojected to view
// space from the depth at its pixel (reprojectPositionToVS), the two horizon
// angles, and the cosine-weighted integral over the normal's slice.  The
// result is stored as r16float.  Texel loads outside the textures read 0
// (robust access); a negative coordinate saturates to 0 when converted to
// u32, as WGSL's conversion does.  Transcendentals (cos, sin, acos, inverse
// square root) are the CUDA library's, so results agree with the oracle to
// a tolerance, not bit for bit.
#define HFB_TU 9
#include <cuda_fp16.h>

#include "hfb_internal.cuh"
#include "hfb_math.cuh"

namespace hfb {
namespace {

constexpr float AO_PI = 3.141592653589793f;
constexpr float AO_HALF_PI = 1.5707963267948966f;
constexpr float AO_Z_NEAR = 0.01f;   // camera.projection.near
constexpr float AO_Z_FAR = 100.0f;   // camera.projection.far

struct AoCtx {
  const float* depth;
  uint32_t W, H;
  float vw, vh;
  const float* pinv;  // projMatrixInv
};

__device__ __forceinline__ uint32_t toU32(float v) { return f2u(v); }  // saturating, as WGSL u32(f32)

__device__ __forceinline__ float loadDepth(const AoCtx& a, float px, float py) {
  const uint32_t x = toU32(px), y = toU32(py);
  return x < a.W && y < a.H ? __ldg(HFB_G(&a.depth[(size_t)y * a.W + x])) : 0.0f;
}

// linearizeDepth, linearDepth.wgsl.ts:9-23
__device__ __forceinline__ float linearizeDepth(float d) {
  return fmul(AO_Z_NEAR, AO_Z_FAR) / fadd(AO_Z_FAR, fmul(fsub(AO_Z_NEAR, AO_Z_FAR), d));
}

// reprojectPositionToVS, gtao.wgsl.ts:23-39
__device__ __forceinline__ f3 reproject(const AoCtx& a, float px, float py) {
  const float d = loadDepth(a, px, py);
  const float x = fsub(fmul(px / a.vw, 2.0f), 1.0f), y = fsub(fmul(py / a.vh, 2.0f), 1.0f);
  const f4 c = m4v(a.pinv, mk4(x, y, d, 1.0f));
  return mk3(c.x / c.w, c.y / c.w, linearizeDepth(d));
}

__device__ __forceinline__ float roundF(float v) { return v < 0.5f ? floorf(v) : ceilf(v); }  // round_f

__device__ __forceinline__ float falloff(float dist, float s2, float e2) {  // gtaoFalloff
  return fmul(2.0f, sat(fsub(dist, s2) / fsub(e2, s2)));
}

__device__ __forceinline__ f3 decodeOct(float fx0, float fy0) {  // decodeOctahedronNormal
  const float fx = fsub(fmul(fx0, 2.0f), 1.0f), fy = fsub(fmul(fy0, 2.0f), 1.0f);
  f3 n = mk3(fx, fy, fsub(fsub(1.0f, fabsf(fx)), fabsf(fy)));
  const float t = sat(-n.z);
  n.x = n.x >= 0.0f ? fsub(n.x, t) : fadd(n.x, t);
  n.y = n.y >= 0.0f ? fsub(n.y, t) : fadd(n.y, t);
  return norm3(n);
}

__device__ float gtao(const HfbUniforms& U, const AoCtx& a, float px, float py, f3 normalWS) {
  const auto& P = U.ao;
  const f3 posVS = reproject(a, px, py);
  f3 nVS = xyz(m4v(U.viewMatrix.m, mk4(normalWS.x, normalWS.y, normalWS.z, 1.0f)));
  nVS.z = -nVS.z;
  const f3 toCam = norm3(mk3(-posVS.x, -posVS.y, -posVS.z));
  if (posVS.z >= fmul(0.999f, AO_Z_FAR)) return 0.0f;
  const float nSteps = (float)P.numSteps;
  const float radius = fmaxf(nSteps, fmul(P.radius, posVS.z / AO_Z_FAR));
  const float stepSize = radius / nSteps;
  float ao = 0.0f;
  const float rotJitter =
      fmul(AO_PI, fractf(fmul(52.9829189f, fractf(fadd(fmul(px, 0.06711056f), fmul(py, 0.00583715f))))));
  const float jitterMod = fmul(fadd(px, py), 0.25f);
  const float radiusJitter = fmul(fmul(fractf(jitterMod), stepSize), 0.25f);
  for (uint32_t i = 0; i < P.numDirections; i++) {
    float phi = fadd(fmul((float)i, AO_PI / (float)P.numDirections), fmul(P.directionOffset, AO_PI));
    phi = fadd(phi, rotJitter);
    float step = fadd(1.0f, fmul(0.25f, stepSize));
    step = fadd(step, radiusJitter);
    const float dx = cosf(phi), dy = sinf(phi);
    float h1 = -1.0f, h2 = -1.0f;
    for (uint32_t j = 0; j < P.numSteps; j++) {
      const float ox = roundF(fmul(dx, step)), oy = roundF(fmul(dy, step));
      {
        const f3 s = reproject(a, fadd(px, ox), fadd(py, oy));
        const f3 ws = sub3(s, posVS);
        const float d2 = len3(ws);
        const float c = fmul(dot3(ws, toCam), rsqrtf(d2));
        h1 = fmaxf(h1, fsub(c, falloff(d2, P.falloffStart2, P.falloffEnd2)));
      }
      {
        const f3 s = reproject(a, fsub(px, ox), fsub(py, oy));
        const f3 ws = sub3(s, posVS);
        const float d2 = len3(ws);
        const float c = fmul(dot3(ws, toCam), rsqrtf(d2));
        h2 = fmaxf(h2, fsub(c, falloff(d2, P.falloffStart2, P.falloffEnd2)));
      }
      step = fadd(step, stepSize);
    }
    h1 = acosf(h1);
    h2 = acosf(h2);
    const f3 dir = mk3(dx, dy, 0.0f);
    const f3 bit = norm3(cross3(dir, toCam));
    const f3 tng = cross3(toCam, bit);
    const f3 nx = sub3(nVS, mul3s(bit, dot3(nVS, bit)));
    const float nnx = len3(nx);
    const float nnxInv = 1.0f / fadd(nnx, 1e-6f);
    const float cosxi = fmul(dot3(nx, tng), nnxInv);
    const float gamma = fsub(acosf(cosxi), AO_HALF_PI);
    const float cosgamma = fmul(dot3(nx, toCam), nnxInv);
    const float singamma2 = fmul(-2.0f, cosxi);
    h1 = fadd(gamma, fmaxf(fsub(-h1, gamma), -AO_HALF_PI));
    h2 = fadd(gamma, fminf(fsub(h2, gamma), AO_HALF_PI));
    const float t1 = fsub(fadd(fmul(h1, singamma2), cosgamma), cosf(fsub(fmul(2.0f, h1), gamma)));
    const float t2 = fsub(fadd(fmul(h2, singamma2), cosgamma), cosf(fsub(fmul(2.0f, h2), gamma)));
    ao = fadd(ao, fmul(fmul(nnx, 0.25f), fadd(t1, t2)));
  }
  return ao / (float)P.numDirections;
}

__global__ void __launch_bounds__(128)
gtaoKernel(const HfbUniforms U, const float* __restrict__ depth, const float2* __restrict__ normals, uint32_t aoW,
           uint32_t aoH, float scale, float* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= aoW * aoH) return;
  AoCtx a;
  a.depth = depth;
  a.W = f2u(U.viewport.x);
  a.H = f2u(U.viewport.y);
  a.vw = U.viewport.x;
  a.vh = U.viewport.y;
  a.pinv = U.projMatrixInv.m;
  const float hx = fadd((float)(i % aoW), 0.5f), hy = fadd((float)(i / aoW), 0.5f);
  const float px = hx / scale, py = hy / scale;
  const uint32_t nx = toU32(px), ny = toU32(py);
  const float2 no = nx < a.W && ny < a.H ? __ldg(HFB_G(&normals[(size_t)ny * a.W + nx])) : make_float2(0.f, 0.f);
  const float v = gtao(U, a, px, py, decodeOct(no.x, no.y));
  *HFB_G(&out[i]) = __half2float(__float2half_rn(v));  // the r16float AO texture
}

}  // namespace

uint32_t aoExtent(float viewport, float scale) { return (uint32_t)ceilf(viewport * scale); }

cudaError_t launchGtao(HfbCtx* c, const HfbUniforms& u, const float* depth, const float* normals, float scale,
                       float* ao) {
  HFB_CHECK_BIND(c);
  const uint32_t aoW = aoExtent(u.viewport.x, scale), aoH = aoExtent(u.viewport.y, scale);
  const uint32_t n = aoW * aoH;
  if (n == 0) return cudaSuccess;
  gtaoKernel<<<divCeil(n, 128u), 128, 0, c->stream>>>(u, depth, (const float2*)normals, aoW, aoH,
                                                       scale, ao);
  HFB_AFTER_LAUNCH(c, "gtaoKernel");
  c->launches += 1;
  return cudaGetLastError();
}

}  // namespace hfb
