// Simulation passes: GridPreSimPass, HairSimIntegrationPass, GridPostSimPass.
//
// Reference WGSL: src/passes/simulation/{gridPreSimPass,hairSimIntegrationPass,
// gridPostSimPass}.wgsl.ts with shaderImpl/{integration,constraints,
// collisions}.wgsl.ts and grids/*.wgsl.ts.  All arithmetic follows the fixed
// fp32 order of hfb_math.cuh, so results are reproducible run to run; the
// grid splat is integer (i32 fixed point, wrapping adds), hence order-free.
#define HFB_TU 1
#include <algorithm>
#include <atomic>

#include "hfb_internal.cuh"
#include "hfb_math.cuh"

namespace hfb {
namespace {

constexpr float GRID_MUL = 1000000.0f;  // GRID_FLOAT_TO_U32_MUL, grids.wgsl.ts:3
// SDF_SAMPLE_GRAD_OFFSET = SDF_CELL_SIZE * 0.1, collisions.wgsl.ts:23-24
// (abstract-float constant expression, rounded once to f32)
constexpr float SDF_GRAD_OFFSET = (float)(0.0033918858971446753 * 0.1);
constexpr float FLOAT_EPSILON = 1e-7f;

__device__ __forceinline__ int32_t gridEncode(float v) { return f2i(fmul(v, GRID_MUL)); }

// Division by the constants 1e6 and 3 as a correctly rounded multiplication
// by the reciprocal, RN(x * Ch + RN(x * Cl)) with Ch + Cl the reciprocal split
// into two floats (Brisebarre and Muller, "Correctly rounded multiplication by
// arbitrary precision constants", IEEE Trans. Computers 57(2), 2008): one
// multiply and one FMA instead of an IEEE division.  For these two constants
// it gives the IEEE quotient x / d bit for bit for every finite x with
// |x| >= 2^-92 (d = 1e6) and |x| > 2^-123 (d = 3); hfb_check_constant_division
// compares it with the device's division over all 2^32 inputs.
constexpr float RCP_1E6_HI = 0x1.0c6f7ap-20f, RCP_1E6_LO = 0x1.6bdb1ap-49f;
constexpr float RCP_3_HI = 0x1.555556p-2f, RCP_3_LO = -0x1.555556p-27f;
__device__ __forceinline__ float mulRcp(float x, float hi, float lo) { return __fmaf_rn(x, hi, fmul(x, lo)); }

// (float)v / 1e6: a converted i32 is 0 or at least 1 in magnitude
__device__ __forceinline__ float gridDecode(int32_t v) { return mulRcp((float)v, RCP_1E6_HI, RCP_1E6_LO); }

__device__ __forceinline__ float divBy3(float x) {
  const float a = fabsf(x);
  return a > 0x1p-123f && a < INFINITY ? mulRcp(x, RCP_3_HI, RCP_3_LO) : x / 3.0f;
}
__device__ __forceinline__ f3 div3sBy3(f3 v) { return {divBy3(v.x), divBy3(v.y), divBy3(v.z)}; }

__device__ __forceinline__ uint32_t gridIdx(uint32_t G, uint32_t x, uint32_t y, uint32_t z) {
  return clampu(z, 0u, G - 1u) * G * G + clampu(y, 0u, G - 1u) * G + clampu(x, 0u, G - 1u);
}

struct GridCo {
  uint32_t mn[3], mx[3];
  f3 p;
};

// _getGridCell, grids.wgsl.ts:43-56
__device__ __forceinline__ GridCo gridCell(uint32_t G, f3 bmin, f3 bmax, f3 p) {
  f3 t = sat3(div3(sub3(p, bmin), sub3(bmax, bmin)));
  float g = (float)(G - 1u);
  GridCo r;
  r.p = mul3s(t, g);
  r.mn[0] = f2u(floorf(r.p.x)); r.mn[1] = f2u(floorf(r.p.y)); r.mn[2] = f2u(floorf(r.p.z));
  r.mx[0] = f2u(ceilf(r.p.x));  r.mx[1] = f2u(ceilf(r.p.y));  r.mx[2] = f2u(ceilf(r.p.z));
  return r;
}

// _getGridCellWeights, grids.wgsl.ts:58-66
__device__ __forceinline__ f3 cellWeights(uint32_t x, uint32_t y, uint32_t z, f3 p) {
  return {clampf(fsub(1.0f, fabsf(fsub(p.x, (float)x))), 0.0f, 1.0f),
          clampf(fsub(1.0f, fabsf(fsub(p.y, (float)y))), 0.0f, 1.0f),
          clampf(fsub(1.0f, fabsf(fsub(p.z, (float)z))), 0.0f, 1.0f)};
}

// sampleSDFCollider (sdfCollider.ts:36-44) with the linear / clamp-to-edge
// sampler of sdfUtils.ts:33-42, as an exact fp32 trilinear filter with texel
// centres at (i + 0.5) / D.
__device__ __forceinline__ float sampleSDF(const float* __restrict__ sdf, uint32_t D, f3 bmin, f3 bmax, f3 p) {
  f3 t = sat3(div3(sub3(p, bmin), sub3(bmax, bmin)));
  float fD = (float)D;
  float u = fsub(fmul(t.x, fD), 0.5f), v = fsub(fmul(t.y, fD), 0.5f), w = fsub(fmul(t.z, fD), 0.5f);
  float fu = floorf(u), fv = floorf(v), fw = floorf(w);
  float ax = fsub(u, fu), ay = fsub(v, fv), az = fsub(w, fw);
  int m = (int)D - 1;
  int x0 = (int)fu, y0 = (int)fv, z0 = (int)fw;
  int x1 = min(max(x0 + 1, 0), m), y1 = min(max(y0 + 1, 0), m), z1 = min(max(z0 + 1, 0), m);
  x0 = min(max(x0, 0), m); y0 = min(max(y0, 0), m); z0 = min(max(z0, 0), m);
  const size_t DD = (size_t)D * D;
  auto T = [&](int x, int y, int z) { return __ldg(HFB_G(sdf + (size_t)z * DD + (size_t)y * D + x)); };
  float c00 = mixf(T(x0, y0, z0), T(x1, y0, z0), ax);
  float c10 = mixf(T(x0, y1, z0), T(x1, y1, z0), ax);
  float c01 = mixf(T(x0, y0, z1), T(x1, y0, z1), ax);
  float c11 = mixf(T(x0, y1, z1), T(x1, y1, z1), ax);
  return mixf(mixf(c00, c10, ay), mixf(c01, c11, ay), az);
}

__device__ __forceinline__ f3 gridMin(const HfbSimUniforms& u) {
  return mk3(u.gridData.boundsMin.x, u.gridData.boundsMin.y, u.gridData.boundsMin.z);
}
__device__ __forceinline__ f3 gridMax(const HfbSimUniforms& u) {
  return mk3(u.gridData.boundsMax[0], u.gridData.boundsMax[1], u.gridData.boundsMax[2]);
}

// ---------------------------------------------------------------------------
// GridPreSimPass.main, gridPreSimPass.wgsl.ts:38-159 (one thread per node)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void gridPreSimBody(const HfbSimUniforms& u, uint32_t G, const int4* __restrict__ dv,
                                               float4* __restrict__ gw, const float* __restrict__ sdf, uint32_t D,
                                               uint32_t id) {
  if (id >= G * G * G) return;
  uint32_t z = id / (G * G);
  uint32_t idXY = id - z * G * G;
  uint32_t y = idXY / G, x = idXY % G;
  f3 gmin = gridMin(u), gmax = gridMax(u);
  f3 cell = div3s(sub3(gmax, gmin), (float)(G - 1u));
  f3 pos = add3(gmin, mul3(cell, mk3((float)x, (float)y, (float)z)));
  f3 smin = mk3(u.sdf.boundsMin.x, u.sdf.boundsMin.y, u.sdf.boundsMin.z);
  f3 smax = mk3(u.sdf.boundsMax.x, u.sdf.boundsMax.y, u.sdf.boundsMax.z);
  // getWindStrength, :89-108
  float wind;
  float d = sampleSDF(sdf, D, smin, smax, pos);
  if (d < 0.0f) {
    wind = 0.0f;
  } else {
    f3 nd = norm3(mk3(u.wind.x, u.wind.y, u.wind.z));
    f3 toward = mk3(-nd.x, -nd.y, -nd.z);
    f3 rp = add3(pos, mul3s(mul3s(toward, d), u.windColisionTraceOffset));
    wind = sampleSDF(sdf, D, smin, smax, rp) < 0.0f ? 0.5f : 1.0f;
  }
  // getDensityGradient, :111-159
  uint32_t idx0 = gridIdx(G, x, y, z);
  float d0 = gridDecode(__ldg(HFB_G(&dv[idx0].w)));
  f3 g = mk3(0.0f, 0.0f, 0.0f);
  const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
#pragma unroll
  for (int k = 0; k < 6; k++) {
    int ox = (int)x + off[k][0], oy = (int)y + off[k][1], oz = (int)z + off[k][2];
    f3 r = mk3(0.0f, 0.0f, 0.0f);
    if (!(ox < 0 || oy < 0 || oz < 0)) {
      uint32_t idxO = gridIdx(G, (uint32_t)ox, (uint32_t)oy, (uint32_t)oz);
      if (idxO != idx0) {
        float dO = gridDecode(__ldg(HFB_G(&dv[idxO].w)));
        float m = fmaxf(fsub(d0, dO), 0.0f);
        r = mul3s(mk3((float)off[k][0], (float)off[k][1], (float)off[k][2]), m);
      }
    }
    g = add3(g, r);
  }
  *HFB_G(&gw[idx0]) = make_float4(g.x, g.y, g.z, wind);
}

__global__ void __launch_bounds__(256) gridPreSimKernel(const HfbSimUniforms u, uint32_t G, const int4* __restrict__ dv,
                                                        float4* __restrict__ gw, const float* __restrict__ sdf,
                                                        uint32_t D) {
  gridPreSimBody(u, G, dv, gw, sdf, D, blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// HairSimIntegrationPass.main, hairSimIntegrationPass.wgsl.ts:79-273
//
// A block holds NB strands' points in shared memory, laid out
// [strand][point + 1]: one thread per strand walks the Gauss-Seidel chains
// (length and local shape must stay sequential along the strand, as in the
// reference), and the whole block runs the per-point phases (Verlet and
// forces, global shape, sphere and SDF collisions) and the coalesced loads
// and stores.  The padding makes both access patterns conflict-free.
//
// The chains are latency-bound (each step waits on the last: an IEEE square
// root and division per step), so what sets the pass's speed is how many
// chains an SM walks at once, and shared memory is what bounds that.  Only
// the points live there (16 B each): the triangle-bending constants and
// initial tangents the local chain reads are written, in the Verlet phase,
// over the block's own points of the PREV buffer -- each thread reads its
// point's previous position first, and nothing else reads those addresses
// until the final positions overwrite them -- and the segment lengths are
// read from their buffer, four at a time where a strand's row is 16-byte
// aligned; the chains load both ahead of the steps that use them.  A block of
// 128 threads holds 2,048 points (64 strands of 32, 128 of 16), six blocks
// per SM: 384 strands of 32 points in flight per SM, three chain warps per
// scheduler.
// ---------------------------------------------------------------------------
constexpr uint32_t SIM_THREADS = 128;        // threads per block of the single-instance kernel
constexpr uint32_t SIM_BATCH_THREADS = 128;  // and of the batched one (6 blocks per SM)


// p + z for z a signed zero whose sign is that of c xor the bit in s: p itself
// unless p is -0 and z is +0
__device__ __forceinline__ void zeroSum(float& p, float c, uint32_t s) {
  if (__float_as_uint(p) == 0x80000000u && ((__float_as_uint(c) ^ s) & 0x80000000u) == 0u) p = 0.0f;
}

// Verlet step of one point with the grid forces (:125-162, integration.wgsl.ts:8-28)
__device__ __forceinline__ float4 verletPoint(const HfbSimUniforms& u, uint32_t G, f3 gmin, f3 gmax,
                                              uint32_t strand, f4 posNow, f4 posPrev,
                                              const int4* __restrict__ dv, const float4* __restrict__ gw) {
  f3 force = mk3(0.0f, -u.gravity, 0.0f);
  const f3 pn = xyz(posNow);
  // _getGridDensityGradAndWind + _getGridDensityVelocity (same cell, two grids)
  GridCo co = gridCell(G, gmin, gmax, pn);
  f3 grad = mk3(0.f, 0.f, 0.f), vel = mk3(0.f, 0.f, 0.f);
  float windStr = 0.0f, dens = 0.0f;
  for (uint32_t z = co.mn[2]; z <= co.mx[2]; z++)
    for (uint32_t y = co.mn[1]; y <= co.mx[1]; y++)
      for (uint32_t x = co.mn[0]; x <= co.mx[0]; x++) {
        f3 w = cellWeights(x, y, z, co.p);
        float wl = len3(w);
        uint32_t idx = gridIdx(G, x, y, z);
        float4 a = __ldg(HFB_G(&gw[idx]));
        grad = add3(grad, mul3(w, mk3(a.x, a.y, a.z)));
        windStr = fadd(windStr, fmul(wl, a.w));
        int4 b = __ldg(HFB_G(&dv[idx]));
        vel = add3(vel, mul3(w, mk3(gridDecode(b.x), gridDecode(b.y), gridDecode(b.z))));
        dens = fadd(dens, fmul(wl, gridDecode(b.w)));
      }
  float timer = fadd(fmul((float)u.frameIdx, 0.73f), fmul(u.windPhaseOffset, (float)strand));
  float windJitter = fractf(fmul(timer, u.windStrengthFrequency));
  float jitterDelta = mixf(fmul(-0.5f, u.windStrengthJitter), fmul(0.5f, u.windStrengthJitter), windJitter);
  float jitterStr = fadd(1.0f, jitterDelta);
  float windCellStr = sat(mixf(u.windStrengthLull, 1.0f, windStr));
  force = add3(force, mul3s(mk3(u.wind.x, u.wind.y, u.wind.z),
                            fabsf(fmul(fmul(u.wind.w, jitterStr), windCellStr))));
  force = add3(force, mul3s(grad, u.volumePreservation));
  f3 gridDisp = dens > 0.0f ? div3s(vel, dens) : mk3(0.f, 0.f, 0.f);
  float dt = u.deltaTime;
  f3 pd = sub3(pn, xyz(posPrev));
  f3 fpd = mix3(pd, gridDisp, u.friction);
  f3 nxt = add3(add3(pn, fpd), mul3s(mul3s(force, dt), dt));
  f3 r = mix3(xyz(posPrev), nxt, posNow.w);
  return make_float4(r.x, r.y, r.z, posNow.w);
}

// applyCollisionsSphere, collisions.wgsl.ts:4-20: pushes pos out of the sphere by kColl.
__device__ __forceinline__ void sphereCollide(float4& pos, const f4 sph, float kColl, bool kCollFinite) {
  f3 v = mk3(fsub(pos.x, sph.x), fsub(pos.y, sph.y), fsub(pos.z, sph.z));
  const float l = len3(v);
  float dist = fsub(l, sph.w);
  float dts = fmaxf(0.0f, -dist);
  if (dts == 0.0f && l > 0.0f && l < INFINITY && kCollFinite) {
    // outside the sphere the correction (v / l) * dts * kColl is a signed zero, the sign
    // of v's component times those of dts and kColl; adding it changes only a -0
    // coordinate, into +0 when the zero is +0
    const uint32_t sz = (__float_as_uint(dts) ^ __float_as_uint(kColl)) & 0x80000000u;
    zeroSum(pos.x, v.x, sz); zeroSum(pos.y, v.y, sz); zeroSum(pos.z, v.z, sz);
  } else {
    f3 d = mul3s(mul3s(norm3(v), dts), kColl);
    pos.x = fadd(pos.x, d.x); pos.y = fadd(pos.y, d.y); pos.z = fadd(pos.z, d.z);
  }
}

// applyCollisionsSdf, collisions.wgsl.ts:23-61, given the distance d sampled at q (pos's xyz).
__device__ __forceinline__ void sdfPush(float4& pos, const f3 q, float d, const float* __restrict__ sdf, uint32_t D,
                                        const f3 smin, const f3 smax, float sdfOffset, float kSdf) {
  float dOff = fadd(d, sdfOffset);
  if (!(dOff >= 0.0f)) {
    const float o = SDF_GRAD_OFFSET;
    f3 cd;
    cd.x = sampleSDF(sdf, D, smin, smax, add3(q, mk3(fmul(o, 1.0f), fmul(o, 0.0f), fmul(o, 0.0f))));
    cd.y = sampleSDF(sdf, D, smin, smax, add3(q, mk3(fmul(o, 0.0f), fmul(o, 1.0f), fmul(o, 0.0f))));
    cd.z = sampleSDF(sdf, D, smin, smax, add3(q, mk3(fmul(o, 0.0f), fmul(o, 0.0f), fmul(o, 1.0f))));
    cd = sub3(cd, mk3(d, d, d));
    f3 corr = mul3s(norm3(cd), -dOff);
    f3 dd = mul3s(corr, kSdf);
    pos.x = fadd(pos.x, dd.x); pos.y = fadd(pos.y, dd.y); pos.z = fadd(pos.z, dd.z);
  }
}

// One step of the length chain (applyConstraint_length, constraints.wgsl.ts:5-28):
// segment j between a (point j, carried in registers) and point j + 1 of the
// staged strand w; writes point j and carries point j + 1 on in a.
__device__ __forceinline__ void lengthStep(float4* w, uint32_t j, float4& a, float expected, float kLen) {
  float4 b = w[j + 1u];
  const float w0 = a.w, w1 = b.w;
  f3 tng = mk3(fsub(b.x, a.x), fsub(b.y, a.y), fsub(b.z, a.z));
  float actual = len3(tng);
  float corr = fsub(1.0f, expected / actual);
  // two movable points (the common case) make the divisor exactly 2: a halving, exact as a product
  const float num = fmul(corr, kLen), den = fadd(fadd(w0, w1), FLOAT_EPSILON);
  float df = den == 2.0f ? fmul(num, 0.5f) : num / den;
  f3 delta = mul3s(tng, df);
  a.x = fadd(a.x, fmul(delta.x, w0)); a.y = fadd(a.y, fmul(delta.y, w0)); a.z = fadd(a.z, fmul(delta.z, w0));
  b.x = fsub(b.x, fmul(w1, delta.x)); b.y = fsub(b.y, fmul(w1, delta.y)); b.z = fsub(b.z, fmul(w1, delta.z));
  w[j] = a;
  a = b;
}

template <uint32_t NT>
__device__ __forceinline__ void simIntegrateBody(const HfbSimUniforms& u, uint32_t S, uint32_t P, uint32_t G,
                                                 float4* __restrict__ prev, const float4* __restrict__ now,
                                                 const float4* __restrict__ initial, const float* __restrict__ segLen,
                                                 const int4* __restrict__ dv, const float4* __restrict__ gw,
                                                 const float* __restrict__ sdf, uint32_t D, float4* simSmem,
                                                 uint32_t blk, uint32_t NB) {
  const uint32_t R = P + 1u;  // row stride (padded)
  float4* wk = simSmem;                                   // [NB][R] positions
  float* att = reinterpret_cast<float*>(wk + NB * R);     // [P] global-shape attenuation of point index j
  const uint32_t tid = threadIdx.x;
  const uint32_t s0 = blk * NB;
  const uint32_t nStr = min(NB, S - s0);
  const uint32_t nPts = nStr * P;
  const f3 gmin = gridMin(u), gmax = gridMax(u);
  // first point matchInitialTangent moves: the triplet loop ends at P - 3
  const uint32_t jTan = P >= 3u ? P - 3u : 0u;
  // the block's points of the PREV buffer: read once by the Verlet phase, then
  // the chain constants of each point, then the new positions
  float4* const lcg = prev + (size_t)s0 * P;

  // --- Verlet + forces and the chain constants, point-parallel ---
#pragma unroll 2
  for (uint32_t i = tid; i < nPts; i += NT) {
    const uint32_t ls = i / P, pt = i - ls * P;
    const size_t gi = (size_t)s0 * P + i;
    const f4 posNow = ld4(__ldg(HFB_G(&now[gi])));
    wk[ls * R + pt] = pt == 0u ? make_float4(posNow.x, posNow.y, posNow.z, posNow.w)
                               : verletPoint(u, G, gmin, gmax, s0 + ls, posNow, ld4(*HFB_G(&prev[gi])), dv, gw);
    const float4 i0 = __ldg(HFB_G(&initial[gi]));
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (pt + 3u < P) {  // applyConstraint_localShape constants (constraints.wgsl.ts:54-99)
      const float4 i1 = __ldg(HFB_G(&initial[gi + 1u])), i2 = __ldg(HFB_G(&initial[gi + 2u]));
      f3 cI = div3sBy3(add3(add3(mk3(i0.x, i0.y, i0.z), mk3(i1.x, i1.y, i1.z)), mk3(i2.x, i2.y, i2.z)));
      const float h0 = len3(sub3(cI, mk3(i1.x, i1.y, i1.z)));
      const float wT = fadd(fadd(i0.w, fmul(2.0f, i1.w)), i2.w);
      c = make_float4(h0, fmul(i0.w / wT, 2.0f), fmul(i1.w / wT, -4.0f), fmul(i2.w / wT, 2.0f));
    } else if (pt >= jTan && pt >= 1u) {  // applyConstraint_matchInitialTangent (:100-120)
      const float4 im = __ldg(HFB_G(&initial[gi - 1u]));
      c = make_float4(fsub(i0.x, im.x), fsub(i0.y, im.y), fsub(i0.z, im.z), 0.0f);
    }
    *HFB_G(&prev[gi]) = c;  // over the previous position this thread has just read
  }
  for (uint32_t j = tid; j < P; j += NT) {  // applyConstraint_global's attenuation (constraints.wgsl.ts:31-49)
    const float x = (float)j / (float)(P - 1u);
    att[j] = fsub(1.0f, sat(fsub(x, u.globalConstrExtent) / u.globalConstrFade));
  }
  // i / P for the block's points (i < NB * P <= 2048, P <= 256): floor(i * ceil(2^32 / P) / 2^32)
  // is exact there, the error i * (ceil(2^32 / P) * P - 2^32) < 2048 * 256 being far below 2^32
  const uint32_t divP = (uint32_t)((0x100000000ull + P - 1u) / P);
  __syncthreads();  // also makes the constants in PREV visible to the block's chain threads

  const uint32_t iters = u.constraintIterations;
  const f3 smin = mk3(u.sdf.boundsMin.x, u.sdf.boundsMin.y, u.sdf.boundsMin.z);
  const f3 smax = mk3(u.sdf.boundsMax.x, u.sdf.boundsMax.y, u.sdf.boundsMax.z);
  const float sdfOffset = u.sdf.boundsMax.w;
  const f4 sph = mk4(u.collisionSphere.x, u.collisionSphere.y, u.collisionSphere.z, u.collisionSphere.w);
  const float kLen = u.stiffnessLengthConstr;
  // a strand's lengths load as float4s when its row starts on a 16-byte boundary
  const bool len4 = (P & 3u) == 0u && (reinterpret_cast<uintptr_t>(segLen) & 15u) == 0u;
  const float kGlob = u.stiffnessGlobalConstr / (float)iters;
  const float kLoc = u.stiffnessLocalConstr / (float)iters;
  const float kColl = u.stiffnessCollisions / (float)iters;
  const bool kCollFinite = fabsf(kColl) < INFINITY;
  const float kSdf = u.stiffnessSDF / (float)iters;
  for (uint32_t it = 0; it < iters; it++) {
    // length constraint (Gauss-Seidel), :176-190, constraints.wgsl.ts:5-28
    for (uint32_t ls = tid; ls < nStr; ls += NT) {
      float4* w = wk + ls * R;
      const float* L = segLen + (size_t)(s0 + ls) * P;
      float4 a = w[0];
      if (len4) {
        // the lengths of steps 4g .. 4g + 3 in one 16-byte load, the next group's issued
        // before this group's steps: four to seven steps ahead
        const float4* L4 = reinterpret_cast<const float4*>(L);
        const uint32_t NG = P >> 2;
        float4 cur = __ldg(HFB_G(&L4[0]));
        for (uint32_t g = 0; g < NG; g++) {
          const float4 nxt = g + 1u < NG ? __ldg(HFB_G(&L4[g + 1u])) : cur;
          const uint32_t j = g << 2;
          lengthStep(w, j, a, cur.x, kLen);
          lengthStep(w, j + 1u, a, cur.y, kLen);
          lengthStep(w, j + 2u, a, cur.z, kLen);
          if (g + 1u < NG) lengthStep(w, j + 3u, a, cur.w, kLen);  // step P - 1 does not exist
          cur = nxt;
        }
      } else {
        float expected = __ldg(HFB_G(&L[0])), nextExpected = __ldg(HFB_G(&L[1]));  // P >= 2
        for (uint32_t j = 0; j + 1u < P; j++) {
          const float nextExpected2 = j + 2u < P ? __ldg(HFB_G(&L[j + 2u])) : 0.0f;  // two steps ahead
          lengthStep(w, j, a, expected, kLen);
          expected = nextExpected;
          nextExpected = nextExpected2;
        }
      }
      w[P - 1u] = a;
    }
    __syncthreads();
    // global shape, :193-206, constraints.wgsl.ts:31-49 (point-parallel)
#pragma unroll 2
    for (uint32_t i = tid; i < nPts; i += NT) {
      const uint32_t ls = __umulhi(i, divP), j = i - ls * P;
      if (j == 0u) continue;
      const float4 pi = __ldg(HFB_G(&initial[(size_t)s0 * P + i]));
      const float k = fmul(kGlob, att[j]);
      float4 p = wk[ls * R + j];
      f3 dvv = mk3(fsub(pi.x, p.x), fsub(pi.y, p.y), fsub(pi.z, p.z));
      f3 d = mul3s(mul3s(dvv, p.w), k);
      p.x = fadd(p.x, d.x); p.y = fadd(p.y, d.y); p.z = fadd(p.z, d.z);
      wk[ls * R + j] = p;
    }
    __syncthreads();
    // local shape (triangle bending, Gauss-Seidel), :209-232, constraints.wgsl.ts:54-120
    for (uint32_t ls = tid; ls < nStr; ls += NT) {
      float4* w = wk + ls * R;
      const float4* C = lcg + (size_t)ls * P;
      uint32_t jj = 0;
      if (P >= 3u) {
        float4 p0 = w[0], p1 = w[1];
        // the constants come from L2 (written this frame): loaded two steps ahead
        float4 cc = *HFB_G(&C[0]), ccNext = *HFB_G(&C[1]);
        for (; jj + 3u < P; jj++) {
          const float4 ccNext2 = *HFB_G(&C[jj + 2u]);  // jj + 2 < P
          float4 p2 = w[jj + 2u];
          f3 c = div3sBy3(add3(add3(mk3(p0.x, p0.y, p0.z), mk3(p1.x, p1.y, p1.z)), mk3(p2.x, p2.y, p2.z)));
          f3 hv = sub3(mk3(p1.x, p1.y, p1.z), c);
          float h = len3(hv);
          f3 delta = mul3s(hv, fsub(1.0f, cc.x / h));
          f3 d0 = mul3s(delta, fmul(kLoc, cc.y)), d1 = mul3s(delta, fmul(kLoc, cc.z)),
             d2 = mul3s(delta, fmul(kLoc, cc.w));
          p0.x = fadd(p0.x, d0.x); p0.y = fadd(p0.y, d0.y); p0.z = fadd(p0.z, d0.z);
          p1.x = fadd(p1.x, d1.x); p1.y = fadd(p1.y, d1.y); p1.z = fadd(p1.z, d1.z);
          p2.x = fadd(p2.x, d2.x); p2.y = fadd(p2.y, d2.y); p2.z = fadd(p2.z, d2.z);
          w[jj] = p0;
          p0 = p1;
          p1 = p2;
          cc = ccNext;
          ccNext = ccNext2;
        }
        w[jj] = p0;
        w[jj + 1u] = p1;
      }
      for (; jj < P; jj++) {  // applyConstraint_matchInitialTangent
        if (jj == 0u) continue;
        const float4 p0 = w[jj - 1u];
        float4 p1 = w[jj];
        const float4 t = *HFB_G(&C[jj]);
        f3 proj = add3(mk3(p0.x, p0.y, p0.z), mk3(t.x, t.y, t.z));
        f3 delta = sub3(proj, mk3(p1.x, p1.y, p1.z));
        f3 d = mul3s(delta, fmul(kLoc, p1.w));
        p1.x = fadd(p1.x, d.x); p1.y = fadd(p1.y, d.y); p1.z = fadd(p1.z, d.z);
        w[jj] = p1;
      }
    }
    __syncthreads();
    // collisions, :236-261, collisions.wgsl.ts:4-61 (point-parallel)
    for (uint32_t i = tid; i < nPts; i += NT) {
      const uint32_t ls = __umulhi(i, divP), j = i - ls * P;
      if (j == 0u) continue;
      float4 pos = wk[ls * R + j];
      sphereCollide(pos, sph, kColl, kCollFinite);
      if (j > 2u) {
        const f3 q = mk3(pos.x, pos.y, pos.z);
        sdfPush(pos, q, sampleSDF(sdf, D, smin, smax, q), sdf, D, smin, smax, sdfOffset, kSdf);
      }
      wk[ls * R + j] = pos;
    }
    __syncthreads();
  }
  // --- write back into the PREV buffer, coalesced (:268-272), over the chain constants ---
  for (uint32_t i = tid; i < nPts; i += NT) {
    const uint32_t ls = i / P, pt = i - ls * P;
    *HFB_G(&prev[(size_t)s0 * P + i]) = wk[ls * R + pt];
  }
  // the staging is rewritten by the CTA's next strands only after batchNext's barrier
}

__global__ void __launch_bounds__(SIM_THREADS, 6)
simIntegrateKernel(const HfbSimUniforms u, uint32_t S, uint32_t P, uint32_t G,
                   float4* __restrict__ prev, const float4* __restrict__ now,
                   const float4* __restrict__ initial, const float* __restrict__ segLen,
                   const int4* __restrict__ dv, const float4* __restrict__ gw,
                   const float* __restrict__ sdf, uint32_t D, uint32_t NB) {
  extern __shared__ float4 simSmem[];
  simIntegrateBody<SIM_THREADS>(u, S, P, G, prev, now, initial, segLen, dv, gw, sdf, D, simSmem, blockIdx.x, NB);
}

// ---------------------------------------------------------------------------
// GridPostSimPass.main, gridPostSimPass.wgsl.ts:45-72 with
// _addGridDensityVelocity, densityVelocityGrid.wgsl.ts:93-124.
//
// Each point adds to the eight corners of its cell, four wrapping i32 adds
// each.  A block takes GP_POINTS points, strand after strand in the order
// strandOrder gives (neighbouring strands next to each other: their points
// share grid nodes), a thread GP_PPT consecutive ones: the points of a run
// in one cell sum their corner values in registers, each run's sums merge
// per grid node in a shared-memory hash table, and each node's four sums
// then go to global memory as one set of atomics.
// Wrapping integer sums do not depend on their order, so the grid is
// bit-exact whatever the strand order and the merge; an update that finds no
// free slot within GP_PROBES goes straight to global memory.
// ---------------------------------------------------------------------------
constexpr uint32_t GP_THREADS = 256;
constexpr uint32_t GP_POINTS = 1024;  // points per block (four per thread)
constexpr uint32_t GP_HASH = 2048;    // slots (power of two)
constexpr uint32_t GP_PROBES = 32;
constexpr uint32_t GP_EMPTY = 0xffffffffu;
constexpr uint32_t GP_PPT = GP_POINTS / GP_THREADS;  // consecutive points per thread
constexpr uint32_t GP_NO_CELL = 0xffffffffu;
constexpr uint32_t GP_BATCH_BLOCKS = 3;  // blocks per SM of the batched kernel (the run sums need registers)

struct GridPostShared {
  uint32_t key[GP_HASH];
  // the four sums of a slot in four arrays: slot h's words sit in bank h mod 32
  // (one uint4 per slot would put slots h and h + 8 in the same banks)
  unsigned vx[GP_HASH], vy[GP_HASH], vz[GP_HASH], vw[GP_HASH];
};

__device__ __forceinline__ void gridPostClear(GridPostShared& sh) {
  for (uint32_t e = threadIdx.x; e < GP_HASH; e += blockDim.x) {
    sh.key[e] = GP_EMPTY;
    sh.vx[e] = 0u; sh.vy[e] = 0u; sh.vz[e] = 0u; sh.vw[e] = 0u;
  }
}

__device__ __forceinline__ void gridPostAdd(GridPostShared& sh, unsigned* __restrict__ dv, uint32_t idx,
                                            uint4 v) {
  uint32_t h = (idx * 2654435761u) >> (32 - 11);  // Fibonacci hash into GP_HASH = 2^11 slots
  for (uint32_t p = 0; p < GP_PROBES; p++) {
    // a slot's key only ever changes from GP_EMPTY to a node index, so a plain read that finds the
    // node (the common case once its first add is in) needs no compare-and-swap
    uint32_t old = *reinterpret_cast<volatile const uint32_t*>(&sh.key[h]);
    if (old == GP_EMPTY) old = atomicCAS(&sh.key[h], GP_EMPTY, idx);
    if (old == GP_EMPTY || old == idx) {
      atomicAdd(&sh.vx[h], v.x);
      atomicAdd(&sh.vy[h], v.y);
      atomicAdd(&sh.vz[h], v.z);
      atomicAdd(&sh.vw[h], v.w);
      return;
    }
    h = (h + 1u) & (GP_HASH - 1u);
  }
  unsigned* c = reinterpret_cast<unsigned*>(HFB_G(reinterpret_cast<uint4*>(dv + 4u * idx)));
  atomicAdd(c + 0, v.x);
  atomicAdd(c + 1, v.y);
  atomicAdd(c + 2, v.z);
  atomicAdd(c + 3, v.w);
}

// Ordered points [blk * GP_POINTS, (blk + 1) * GP_POINTS) of the S * P: the
// ordered point v is point v % P of strand order[v / P].  The table is empty
// on entry and on exit.  All threads of the block call it.
__device__ __forceinline__ void gridPostSimBody(const HfbSimUniforms& u, uint32_t S, uint32_t P, uint32_t G,
                                                const float4* __restrict__ prev, const float4* __restrict__ now,
                                                unsigned* __restrict__ dv, const uint32_t* __restrict__ order,
                                                uint32_t blk, GridPostShared& sh) {
  const uint32_t N = S * P;
  const f3 gmin = gridMin(u), gmax = gridMax(u);
  // a thread's GP_PPT consecutive ordered points: consecutive points that fall in
  // the same cell (mostly neighbours on one strand) add their corner values in
  // registers first (wrapping, as the table and the grid do), and the cell's sums
  // go to the table when the cell changes or the points end -- one set of table
  // adds per run of points
  uint4 acc[8];
  uint32_t c0 = 0, c1 = 0, c2 = 0, cm = GP_NO_CELL;  // the cell being summed; cm: its corner mask
  const uint32_t vb = blk * GP_POINTS + threadIdx.x * GP_PPT;
#pragma unroll 1
  for (uint32_t r = 0; r <= GP_PPT; r++) {
    const uint32_t v = vb + r;
    const bool more = r < GP_PPT && v < N;
    GridCo co;
    f3 vel;
    uint32_t m = GP_NO_CELL;
    if (more) {
      const uint32_t ls = v / P, j = v - ls * P;
      const uint32_t s = order ? min(__ldg(HFB_G(&order[ls])), S - 1u) : ls;
      const size_t i = (size_t)s * P + j;
      const float4 a = __ldg(HFB_G(&prev[i])), b = __ldg(HFB_G(&now[i]));
      const f3 pn = mk3(b.x, b.y, b.z);
      vel = sub3(pn, mk3(a.x, a.y, a.z));
      co = gridCell(G, gmin, gmax, pn);
      // corner k = x + 2y + 4z (offsets from mn) exists when each of its offsets is 0 or mx > mn there
      m = (co.mx[0] > co.mn[0] ? 1u : 0u) | (co.mx[1] > co.mn[1] ? 2u : 0u) | (co.mx[2] > co.mn[2] ? 4u : 0u);
    }
    if (!more || m != cm || co.mn[0] != c0 || co.mn[1] != c1 || co.mn[2] != c2) {
      if (cm != GP_NO_CELL) {
#pragma unroll
        for (uint32_t k = 0; k < 8u; k++)
          if ((k & ~cm) == 0u)
            gridPostAdd(sh, dv, gridIdx(G, c0 + (k & 1u), c1 + ((k >> 1) & 1u), c2 + (k >> 2)), acc[k]);
      }
      if (!more) break;
#pragma unroll
      for (uint32_t k = 0; k < 8u; k++) acc[k] = make_uint4(0u, 0u, 0u, 0u);
      c0 = co.mn[0]; c1 = co.mn[1]; c2 = co.mn[2]; cm = m;
    }
#pragma unroll
    for (uint32_t k = 0; k < 8u; k++) {
      if ((k & ~m) != 0u) continue;
      const uint32_t x = co.mn[0] + (k & 1u), y = co.mn[1] + ((k >> 1) & 1u), z = co.mn[2] + (k >> 2);
      const f3 w = cellWeights(x, y, z, co.p);
      const f3 cv = mul3(vel, w);
      acc[k].x += (unsigned)gridEncode(cv.x);
      acc[k].y += (unsigned)gridEncode(cv.y);
      acc[k].z += (unsigned)gridEncode(cv.z);
      acc[k].w += (unsigned)gridEncode(len3(w));
    }
  }
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < GP_HASH; e += blockDim.x) {
    const uint32_t idx = sh.key[e];
    if (idx == GP_EMPTY) continue;
    const uint4 v = make_uint4(sh.vx[e], sh.vy[e], sh.vz[e], sh.vw[e]);
    unsigned* c = reinterpret_cast<unsigned*>(HFB_G(reinterpret_cast<uint4*>(dv + 4u * idx)));
    atomicAdd(c + 0, v.x);
    atomicAdd(c + 1, v.y);
    atomicAdd(c + 2, v.z);
    atomicAdd(c + 3, v.w);
    sh.key[e] = GP_EMPTY;
    sh.vx[e] = 0u; sh.vy[e] = 0u; sh.vz[e] = 0u; sh.vw[e] = 0u;
  }
  // the next points' adds come after batchNext's barrier, with the table empty
}

__global__ void __launch_bounds__(GP_THREADS)
gridPostSimKernel(const HfbSimUniforms u, uint32_t S, uint32_t P, uint32_t G, const float4* __restrict__ prev,
                  const float4* __restrict__ now, unsigned* __restrict__ dv, const uint32_t* __restrict__ order) {
  __shared__ GridPostShared sh;
  gridPostClear(sh);
  __syncthreads();
  gridPostSimBody(u, S, P, G, prev, now, dv, order, blockIdx.x, sh);
}

// ---- batched: persistent over the virtual blocks of every instance ----
// 5 blocks per SM (48 registers): 0.45 ms against 0.50 at 4 (64 registers) on the 64-instance frame
__global__ void __launch_bounds__(256, 5) gridPreSimBatch(BatchView b, uint32_t G) {
  const uint32_t n = b.hdr->n;
  const uint32_t* row = b.prefix + BK_GRID_PRE * (BATCH_MAX + 1);
  const uint32_t total = row[n];
  __shared__ uint32_t vbNext[2];
  uint32_t vbPar = 0;
  for (uint32_t v = batchNext(b.hdr, BK_GRID_PRE, vbNext, vbPar); v < total; v = batchNext(b.hdr, BK_GRID_PRE, vbNext, vbPar)) {
    const uint32_t i = batchFind(row, n, v);
    const BatchInst& I = b.insts[i];
    gridPreSimBody(I.SU, G, I.dv, I.gw, I.sdf, I.sdfDims, (v - row[i]) * 256u + threadIdx.x);
  }
}

__global__ void __launch_bounds__(SIM_BATCH_THREADS, 6) simIntegrateBatch(BatchView b, uint32_t G) {
  extern __shared__ float4 simSmem[];
  const uint32_t n = b.hdr->n;
  const uint32_t* row = b.prefix + BK_INTEGRATE * (BATCH_MAX + 1);
  const uint32_t total = row[n];
  __shared__ uint32_t vbNext[2];
  uint32_t vbPar = 0;
  for (uint32_t v = batchNext(b.hdr, BK_INTEGRATE, vbNext, vbPar); v < total; v = batchNext(b.hdr, BK_INTEGRATE, vbNext, vbPar)) {
    const uint32_t i = batchFind(row, n, v);
    const BatchInst& I = b.insts[i];
    // integration reads positions[1 - current] (prev) and [current] (now), writes the former
    simIntegrateBody<SIM_BATCH_THREADS>(I.SU, I.S, I.P, G, I.posNew, I.posOld, I.initial, I.segLen, I.dv, I.gw, I.sdf, I.sdfDims,
                     simSmem, v - row[i], simStrandsPerBlock(I.P));
  }
}

__global__ void __launch_bounds__(GP_THREADS, GP_BATCH_BLOCKS) gridPostSimBatch(BatchView b, uint32_t G) {
  __shared__ GridPostShared sh;
  gridPostClear(sh);
  __syncthreads();
  const uint32_t n = b.hdr->n;
  const uint32_t* row = b.prefix + BK_GRID_POST * (BATCH_MAX + 1);
  const uint32_t total = row[n];
  __shared__ uint32_t vbNext[2];
  uint32_t vbPar = 0;
  for (uint32_t v = batchNext(b.hdr, BK_GRID_POST, vbNext, vbPar); v < total; v = batchNext(b.hdr, BK_GRID_POST, vbNext, vbPar)) {
    const uint32_t i = batchFind(row, n, v);
    const BatchInst& I = b.insts[i];
    // after the swap: prev = the old current positions, now = the new ones
    gridPostSimBody(I.SU, I.S, I.P, G, I.posOld, I.posNew, (unsigned*)I.dv, I.gridOrder, v - row[i], sh);
  }
}


// Compares the reciprocal forms above with the IEEE division over all 2^32
// inputs: cnt[0] x / 3 over every non-NaN float, cnt[1] (float)v / 1e6 over
// every i32 v, cnt[2] x / 1e6 over every finite float with |x| >= 2^-92.
__global__ void __launch_bounds__(256) constDivCheckKernel(unsigned long long* __restrict__ cnt) {
  unsigned long long bad3 = 0, badGrid = 0, bad6 = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (1ull << 32); i += stride) {
    const uint32_t bits = (uint32_t)i;
    const float x = __uint_as_float(bits);
    if (x == x) {
      bad3 += __float_as_uint(divBy3(x)) != __float_as_uint(x / 3.0f);
      const float a = fabsf(x);
      if (a >= 0x1p-92f && a < INFINITY)
        bad6 += __float_as_uint(mulRcp(x, RCP_1E6_HI, RCP_1E6_LO)) != __float_as_uint(x / GRID_MUL);
    }
    const int32_t v = (int32_t)bits;
    badGrid += __float_as_uint(gridDecode(v)) != __float_as_uint((float)v / GRID_MUL);
  }
  if (bad3) atomicAdd(&cnt[0], bad3);
  if (badGrid) atomicAdd(&cnt[1], badGrid);
  if (bad6) atomicAdd(&cnt[2], bad6);
}

}  // namespace

cudaError_t launchConstDivCheck(HfbCtx* c, unsigned long long* cnt) {
  HFB_CHECK_BIND(c);
  cudaError_t e = cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned long long), c->stream);
  if (e != cudaSuccess) return e;
  constDivCheckKernel<<<c->smCount * 8u, 256, 0, c->stream>>>(cnt);
  HFB_AFTER_LAUNCH(c, "constDivCheckKernel");
  c->launches += 1;
  return cudaGetLastError();
}

cudaError_t launchGridPreSim(HfbCtx* c, const HfbSimUniforms& u, const int32_t* dv, float* gw,
                             const float* sdf, uint32_t sdfDims) {
  HFB_CHECK_BIND(c);
  uint32_t G = c->cfg.gridDims;
  uint32_t n = G * G * G;
  gridPreSimKernel<<<divCeil(n, 256), 256, 0, c->stream>>>(u, G, (const int4*)dv, (float4*)gw, sdf, sdfDims);
  HFB_AFTER_LAUNCH(c, "gridPreSimKernel");
  c->launches += 1;
  return cudaGetLastError();
}

// The dynamic shared memory limit of a kernel is a setting of the function
// for the whole process (per device), not of a context: contexts with
// different strand lengths would lower it under one another's launches.  It
// is raised once, to what the longest strands need.
static cudaError_t simSmemLimit(const void* fn, int which) {
  static std::atomic<uint64_t> done[2] = {};  // bit d: set on device d
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = 1ull << (dev & 63);
  if (done[which].load() & bit) return cudaSuccess;
  size_t most = 0;
  for (uint32_t P = 2; P <= 256; P++) most = std::max(most, simSmemBytes(P));
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
  if (e == cudaSuccess) done[which].fetch_or(bit);
  return e;
}

cudaError_t launchSimIntegrate(HfbCtx* c, const HfbSimUniforms& u, const HfbHairData& h, float* prev,
                               const float* now, const float* initial, const float* segLen,
                               const int32_t* dv, const float* gw, const float* sdf, uint32_t sdfDims) {
  HFB_CHECK_BIND(c);
  const uint32_t S = h.strandsCount, P = h.pointsPerStrand;
  // one instance alone rarely fills the GPU: its blocks take fewer strands
  // (down to 8) until there are two per SM, so that more chains run at once
  const uint32_t NB = simStrandsPerBlockFor(S, P, (uint32_t)c->smCount);
  const size_t smem = (size_t)NB * (P + 1u) * sizeof(float4) + (size_t)P * 4u;
  cudaError_t e = simSmemLimit((const void*)simIntegrateKernel, 0);
  if (e != cudaSuccess) return e;
  simIntegrateKernel<<<divCeil(S, NB), SIM_THREADS, smem, c->stream>>>(
      u, S, P, c->cfg.gridDims, (float4*)prev, (const float4*)now, (const float4*)initial, segLen,
      (const int4*)dv, (const float4*)gw, sdf, sdfDims, NB);
  HFB_AFTER_LAUNCH(c, "simIntegrateKernel");
  c->launches += 1;
  return cudaGetLastError();
}

cudaError_t launchBatchSim(HfbCtx* c, const BatchView& b, BatchKind k) {
  HFB_CHECK_BIND(c);
  const uint32_t G = c->cfg.gridDims;
  uint32_t& grid = c->batchGrid[k];
  if (k == BK_GRID_PRE) {
    if (!grid) grid = c->smCount * 8u;
    gridPreSimBatch<<<batchLaunchGrid(c, grid), 256, 0, c->stream>>>(b, G);
    HFB_AFTER_LAUNCH(c, "gridPreSimBatch");
  } else if (k == BK_INTEGRATE) {
    const size_t smem = c->simBatchSmem;  // the largest staging any batch of the context has needed
    if (!grid) {
      cudaError_t e = simSmemLimit((const void*)simIntegrateBatch, 1);
      int perSM = 0;
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, simIntegrateBatch, SIM_BATCH_THREADS, smem);
      if (e != cudaSuccess) return e;
      grid = (uint32_t)(perSM > 0 ? perSM : 1) * c->smCount;
    }
    simIntegrateBatch<<<batchLaunchGrid(c, grid), SIM_BATCH_THREADS, smem, c->stream>>>(b, G);
    HFB_AFTER_LAUNCH(c, "simIntegrateBatch");
  } else if (k == BK_GRID_POST) {
    if (!grid) {
      int perSM = 0;
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, gridPostSimBatch, GP_THREADS, 0);
      if (e != cudaSuccess) return e;
      grid = (uint32_t)(perSM > 0 ? perSM : 1) * c->smCount;
    }
    gridPostSimBatch<<<batchLaunchGrid(c, grid), GP_THREADS, 0, c->stream>>>(b, G);
    HFB_AFTER_LAUNCH(c, "gridPostSimBatch");
  } else {
    return cudaErrorInvalidValue;
  }
  c->launches += 1;
  return cudaGetLastError();
}

uint32_t gridPostBlocks(uint32_t points) { return divCeil(points, GP_POINTS); }

cudaError_t launchGridPostSim(HfbCtx* c, const HfbSimUniforms& u, const HfbHairData& h, const float* prev,
                              const float* now, int32_t* dv, const uint32_t* strandOrder) {
  HFB_CHECK_BIND(c);
  uint32_t G = c->cfg.gridDims;
  cudaError_t e = cudaMemsetAsync(dv, 0, (size_t)G * G * G * 16, c->stream);  // clearDensityVelocityBuffer
  if (e != cudaSuccess) return e;
  const uint32_t N = h.strandsCount * h.pointsPerStrand;
  if (N) {
    gridPostSimKernel<<<gridPostBlocks(N), GP_THREADS, 0, c->stream>>>(
        u, h.strandsCount, h.pointsPerStrand, G, (const float4*)prev, (const float4*)now, (unsigned*)dv, strandOrder);
    HFB_AFTER_LAUNCH(c, "gridPostSimKernel");
    c->launches += 1;
  }
  return cudaGetLastError();
}

}  // namespace hfb
