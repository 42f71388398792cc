// Composite + present: HairCombinePass and PresentPass as one CUDA pass.
//
// HairCombinePass (hairCombinePass.wgsl.ts:51-89, pipeline blend state
// hairCombinePass.ts:40-52) draws the fine pass's result over the scene
// colour with src-alpha / one-minus-src-alpha, reading the result buffer
// upside down (fragment row y reads result row H - 1 - y).  PresentPass
// (presentPass.wgsl.ts: main_fs, DISPLAY_MODE_FINAL) then dithers (8x8 Bayer,
// dither.wgsl.ts:26-53), applies the exposure, ACES (aces.wgsl.ts:6-13) with
// saturate, and gamma (pow(c, 1 / gamma)); the swap chain stores unorm8,
// c * 255 rounded to nearest.  Out: RGBA8, row 0 at the top, alpha 255.
#define HFB_TU 8
#include "hfb_internal.cuh"
#include "hfb_math.cuh"

namespace hfb {
namespace {

__constant__ uint8_t kBayer[64] = {0,  32, 8,  40, 2,  34, 10, 42, 48, 16, 56, 24, 50, 18, 58, 26,
                                   12, 44, 4,  36, 14, 46, 6,  38, 60, 28, 52, 20, 62, 30, 54, 22,
                                   3,  35, 11, 43, 1,  33, 9,  41, 51, 19, 59, 27, 49, 17, 57, 25,
                                   15, 47, 7,  39, 13, 45, 5,  37, 63, 31, 55, 23, 61, 29, 53, 21};

__device__ __forceinline__ float aces(float x) {  // doACES_Tonemapping, one channel
  const float num = fmul(x, fadd(fmul(2.51f, x), 0.03f));
  const float den = fadd(fmul(x, fadd(fmul(2.43f, x), 0.59f)), 0.14f);
  return sat(num / den);
}

__device__ __forceinline__ uint8_t unorm8(float c) {  // float -> unorm8, round to nearest
  return (uint8_t)__float2uint_rn(fmul(sat(c), 255.0f));
}

// Pixel i (row-major, row 0 at the top) of one image.
__device__ __forceinline__ void presentPixel(float gamma, float exposure, float ditherStr, uint32_t W, uint32_t H,
                                             const float4* __restrict__ result, const float4* __restrict__ scene,
                                             uchar4* __restrict__ out, uint32_t i) {
  const uint32_t x = i % W, y = i / W;  // y: row from the top
  const float4 src = __ldg(HFB_G(&result[(size_t)(H - 1u - y) * W + x]));
  const float4 dst = scene ? __ldg(HFB_G(&scene[i])) : make_float4(0.f, 0.f, 0.f, 1.f);
  // blend: src * src.a + dst * (1 - src.a)
  const float ia = fsub(1.0f, src.w);
  float c[3] = {fadd(fmul(src.x, src.w), fmul(dst.x, ia)), fadd(fmul(src.y, src.w), fmul(dst.y, ia)),
                fadd(fmul(src.z, src.w), fmul(dst.z, ia))};
  const float dither = fmul((float)kBayer[(y % 8u) * 8u + (x % 8u)] / 63.0f, ditherStr) / 256.0f;
  uint8_t o[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float v = fadd(c[k], dither);
    v = fmul(v, exposure);
    v = aces(v);
    v = powf(v, 1.0f / gamma);
    o[k] = unorm8(v);
  }
  *HFB_G(&out[i]) = make_uchar4(o[0], o[1], o[2], 255);
}

__global__ void __launch_bounds__(256)
presentKernel(float gamma, float exposure, float ditherStr, uint32_t W, uint32_t H, const float4* __restrict__ result,
              const float4* __restrict__ scene, uchar4* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * H) return;
  presentPixel(gamma, exposure, ditherStr, W, H, result, scene, out, i);
}

// Up to PRESENT_BATCH images in one launch, passed by value (48 B each, inside
// the 4 KB of kernel parameters every launch may carry): image k covers the
// launch's pixels [first[k], first[k + 1]).
constexpr uint32_t PRESENT_BATCH = 64;
struct PresentImage {
  float gamma, exposure, dither;
  uint32_t W, H, first;
  const float4* result;
  const float4* scene;
  uchar4* out;
};
struct PresentBatch {
  uint32_t n, total;
  PresentImage im[PRESENT_BATCH];
};
static_assert(sizeof(PresentBatch) <= 4000, "kernel parameters above 4 KB");

__global__ void __launch_bounds__(256) presentBatchKernel(const PresentBatch pb) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < pb.total; g += stride) {
    uint32_t lo = 0, hi = pb.n - 1u;  // the last image whose first pixel is at or before g
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1u) >> 1;
      if (pb.im[mid].first <= g) lo = mid; else hi = mid - 1u;
    }
    const PresentImage& m = pb.im[lo];
    presentPixel(m.gamma, m.exposure, m.dither, m.W, m.H, m.result, m.scene, m.out, g - m.first);
  }
}

}  // namespace

cudaError_t launchPresent(HfbCtx* c, const HfbUniforms& u, uint32_t W, uint32_t H, const float* result,
                          const float* scene, uint8_t* rgba) {
  HFB_CHECK_BIND(c);
  const uint32_t n = W * H;
  if (n == 0) return cudaSuccess;
  presentKernel<<<divCeil(n, 256u), 256, 0, c->stream>>>(u.colorMgmt.x, u.colorMgmt.y, u.colorMgmt.z, W, H,
                                                         (const float4*)result, (const float4*)scene, (uchar4*)rgba);
  HFB_AFTER_LAUNCH(c, "presentKernel");
  c->launches += 1;
  return cudaGetLastError();
}

// Images of at most 2^32 - 1 pixels in all per launch of PRESENT_BATCH; the
// caller has checked every item.
cudaError_t launchPresentBatch(HfbCtx* c, const HfbPresentItem* items, uint32_t n) {
  HFB_CHECK_BIND(c);
  for (uint32_t k0 = 0; k0 < n; k0 += PRESENT_BATCH) {
    PresentBatch pb{};
    uint64_t total = 0;
    for (uint32_t k = k0; k < n && k < k0 + PRESENT_BATCH; k++) {
      const HfbPresentItem& it = items[k];
      const uint32_t W = it.rb->width, H = it.rb->height;
      if ((uint64_t)W * H == 0u) continue;
      if (total + (uint64_t)W * H > 0xffffffffull) return cudaErrorInvalidValue;
      PresentImage& m = pb.im[pb.n++];
      m.gamma = it.uniforms->colorMgmt.x;
      m.exposure = it.uniforms->colorMgmt.y;
      m.dither = it.uniforms->colorMgmt.z;
      m.W = W;
      m.H = H;
      m.first = (uint32_t)total;
      m.result = (const float4*)(it.rb->rasterizerResult + 4);
      m.scene = (const float4*)it.sceneColor;
      m.out = (uchar4*)it.rgba;
      total += (uint64_t)W * H;
    }
    if (pb.n == 0) continue;
    pb.total = (uint32_t)total;
    const uint32_t blocks = divCeil(pb.total, 256u);
    const uint32_t cap = c->smCount * 8u;
    presentBatchKernel<<<blocks < cap ? blocks : cap, 256, 0, c->stream>>>(pb);
    HFB_AFTER_LAUNCH(c, "presentBatchKernel");
    c->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace hfb
