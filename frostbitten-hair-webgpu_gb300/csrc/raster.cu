// Software raster passes: HairTilesPass, HairTileSortPass, HairFinePass.
//
// Reference WGSL: src/passes/swHair/hairTilesPass.wgsl.ts:70-246,
// hairTileSortPass.countTiles.wgsl.ts:21-97, hairTileSortPass.sort.wgsl.ts:35-75,
// hairFinePass.wgsl.ts:41-335 with shaderImpl/{swRasterizeHair,
// processHairSegment,reduceHairSlices,tileUtils}.wgsl.ts and the buffer
// layouts of shared/*.ts.
//
// Tiles pass = 5 kernels:
//   1. tilesRaster   one thread per (strand, segment): project, bound, walk
//                    the covered pixels of every tile of the bounding rect,
//                    emit one (tile-bin, key) record per touched tile; the
//                    head min/max depth atomics and the per-tile counts are
//                    order independent.
//   2. binScan       exclusive prefix of the per-(tile, bin) record counts.
//   3. binScatter    counting-sort scatter of the record keys into CSR order.
//   4. binFinalize   sort each (tile, bin)'s keys ascending and write the
//                    reference's linked list (head -> largest key): a warp
//                    per bin (single instance); in the batched frame 8 lanes
//                    per bin of at most 8 records and a warp per larger bin.
//   5. largeBins     one CTA per bin with more than 1024 records.
// The resulting lists are canonical: they do not depend on atomic order.
#include <cooperative_groups.h>
#include <cuda_fp16.h>
#include <type_traits>

#define HFB_TU 3
#include "hfb_internal.cuh"
#include "hfb_math.cuh"

namespace cg = cooperative_groups;

namespace hfb {
namespace {

constexpr uint32_t INVALID_PTR = 0xffffffffu;
constexpr float F_MAX_U32 = 4294967296.0f;  // f32(MAX_U32)
constexpr uint32_t SMALL_BIN = 32;
constexpr uint32_t MEDIUM_BIN = 1024;
constexpr uint32_t LARGE_SMEM_KEYS = 16384;
constexpr int SCAN_PER_BLOCK = 2048;

struct TileB { uint32_t x0, y0, x1, y1; };

// getTileBoundsPx, tileUtils.wgsl.ts:43-54
__device__ __forceinline__ TileB tileBoundsPx(uint32_t W, uint32_t H, uint32_t TS, uint32_t tx, uint32_t ty) {
  return {clampu(tx * TS, 0u, W - 1u), clampu(ty * TS, 0u, H - 1u), clampu((tx + 1u) * TS, 0u, W - 1u),
          clampu((ty + 1u) * TS, 0u, H - 1u)};
}

__device__ __forceinline__ ProjSeg projectSegment(const HfbUniforms& U, const float4* __restrict__ pos,
                                                  const float4* __restrict__ tan, uint32_t P, uint32_t strand,
                                                  uint32_t seg, f2 size) {
  ProjSeg r;
  f3 cam = mk3(U.cameraPosition.x, U.cameraPosition.y, U.cameraPosition.z);
  size_t i = (size_t)strand * P + seg;
  projectHairPoint(U.modelMatrix.m, U.vpMatrix.m, cam, ld4(__ldg(HFB_G(&pos[i]))), ld4(__ldg(HFB_G(&tan[i]))), size,
                   U.fiberRadius, r.v00, r.v01, r.depthsProj.x, r.depthsProj.y);
  projectHairPoint(U.modelMatrix.m, U.vpMatrix.m, cam, ld4(__ldg(HFB_G(&pos[i + 1]))), ld4(__ldg(HFB_G(&tan[i + 1]))), size,
                   U.fiberRadius, r.v10, r.v11, r.depthsProj.z, r.depthsProj.w);
  return r;
}

__device__ __forceinline__ bool insideQuad(const ProjSeg& s, f2 p) {
  float C0 = edgeFunction(s.v01, s.v00, p);
  float C1 = edgeFunction(s.v11, s.v01, p);
  float C2 = edgeFunction(s.v10, s.v11, p);
  float C3 = edgeFunction(s.v00, s.v10, p);
  return C0 >= 0.0f && C1 >= 0.0f && C2 >= 0.0f && C3 >= 0.0f;
}

// Candidate pixels of one row of a projected segment quad.  The four edge
// functions are linear in x along a row, so the covered interval follows
// from the edge equations: x = a.x + (y - a.y) * slope per edge.  Edges with
// |slope| > 64 (nearly horizontal, ill conditioned) are skipped, which bounds
// the fp32 error of the solved x by ~0.03 px at 4096 px; a 2-pixel margin
// keeps every pixel the exact fp32 edge test accepts inside the candidate
// range -- the exact test still decides each pixel.
struct RowSpan {
  float ax[4], ay[4], slope[4];
  uint32_t lower;  // bit i: edge i bounds x from below (A > 0), else from above
  uint32_t use;    // bit i: edge i is used
  __device__ __forceinline__ void candidates(float y, uint32_t& x0, uint32_t& x1) const {
    float lo = -1e30f, hi = 1e30f;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (!((use >> i) & 1u)) continue;
      float b = ax[i] + (y - ay[i]) * slope[i];
      if ((lower >> i) & 1u) lo = fmaxf(lo, b); else hi = fminf(hi, b);
    }
    if (!(lo <= hi + 4.0f)) { x1 = x0; return; }  // empty row (NaN-safe)
    float l = floorf(lo) - 2.0f, h = ceilf(hi) + 3.0f;
    if (l > (float)x0) x0 = (uint32_t)fminf(l, 4294967040.0f);
    if (h < (float)x1) x1 = h < 0.0f ? 0u : (uint32_t)h;
    if (x1 < x0) x1 = x0;
  }
};

__device__ __forceinline__ RowSpan makeRowSpan(const ProjSeg& s) {
  // edges in the order the test uses: v01->v00, v11->v01, v10->v11, v00->v10
  const f2 a[4] = {s.v01, s.v11, s.v10, s.v00};
  const f2 b[4] = {s.v00, s.v01, s.v11, s.v10};
  RowSpan r;
  r.lower = 0u;
  r.use = 0u;
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float A = b[i].y - a[i].y, Bx = b[i].x - a[i].x;
    r.ax[i] = a[i].x;
    r.ay[i] = a[i].y;
    r.slope[i] = Bx / A;
    if (fabsf(A) * 64.0f >= fabsf(Bx) + 1.0f) r.use |= 1u << i;
    if (A > 0.0f) r.lower |= 1u << i;
    finite = finite && isfinite(a[i].x) && isfinite(a[i].y);
  }
  if (!finite) r.use = 0u;
  return r;
}

// Block-wide exclusive prefix (all threads call; total = block sum).
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* warpSums, uint32_t& total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) warpSums[warp] = x;
  __syncthreads();
  const uint32_t nw = blockDim.x >> 5;
  if (warp == 0) {
    uint32_t s = lane < nw ? warpSums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= (uint32_t)o) s += y;
    }
    if (lane < nw) warpSums[lane] = s;
  }
  __syncthreads();
  total = warpSums[nw - 1];
  uint32_t warpPrefix = warp ? warpSums[warp - 1] : 0u;
  __syncthreads();
  return warpPrefix + x - v;
}

// ---------------------------------------------------------------------------
// 1. tilesRaster: HairTilesPass.main + processTile, hairTilesPass.wgsl.ts:70-238
//
// A block takes TR_SEGS consecutive segments.  The candidate pixels of a
// segment are its bounding rectangle clipped to the pixels the tiles cover
// ([0, W - 1) x [0, H - 1): getTileBoundsPx clamps the tile ends to W - 1 /
// H - 1), each belonging to tile (x / TS, y / TS).  The block then runs:
//   A1  one thread per (segment, candidate pixel) pair: the edge tests;
//       passing pairs are appended to the warp's region of a list;
//   A2  one thread per passing pixel: interpolated depth, the depth test
//       against the scene and, where the bin does not follow from the depth
//       range (binRange), the view-space depth bin, folded into the
//       (segment, tile) accumulators with shared-memory atomics (min / max
//       over an order-preserving u32 image of the depth, min of the bin):
//       the result does not depend on the order;
//   E   one thread per (segment, tile): the record, as processTile stores
//       it (:220-237).
// A segment whose tiles do not fit the block's accumulators is walked by its
// own thread, tile by tile (rasterSegmentSerial).
// ---------------------------------------------------------------------------
constexpr uint32_t TR_SEGS = TILES_RASTER_SEGS;  // segments (and threads) per block
// (segment, tile) accumulators per block and list entries per A1 / A2 round: the
// single-instance kernel keeps more of a large frame's long segments in
// shared memory (768, 2,048: 6 CTAs per SM); the batched one, whose
// instances are smaller, trades them for a seventh CTA (512, 1,024).
constexpr uint32_t TR_SLOTS = 768, TR_CHUNK = 2048;
constexpr uint32_t TR_SLOTS_BATCH = 512, TR_CHUNK_BATCH = 1024;

template <uint32_t TR_SLOTS, uint32_t TR_CHUNK>
struct TrShared {
  float ox[4][TR_SEGS], oy[4][TR_SEGS], ex[4][TR_SEGS], ey[4][TR_SEGS];  // edge tests (insideQuad order)
  float dp[4][TR_SEGS];                                                 // depthsProj
  float qsx[TR_SEGS], qsy[TR_SEGS], qax[TR_SEGS], qay[TR_SEGS], qd2[TR_SEGS], qlse[TR_SEGS], qws[TR_SEGS],
      qwe[TR_SEGS], qd22[TR_SEGS];                                      // QuadConst
  uint32_t cx0[TR_SEGS], cy0[TR_SEGS], cw[TR_SEGS];  // candidate rectangle origin and width
  uint32_t tminx[TR_SEGS], tminy[TR_SEGS], tsx[TR_SEGS];
  float blo[TR_SEGS], bhi[TR_SEGS];  // depth range over which the bin follows from the depth alone
  uint32_t pairBase[TR_SEGS + 1], slotBase[TR_SEGS + 1];
  uint32_t accMin[TR_SLOTS], accMax[TR_SLOTS], accBin[TR_SLOTS];
  uint32_t pass[TR_CHUNK];  // segment | column in the rectangle << 7 | row << 19, one region per warp
  uint32_t warpSums[32];
  uint32_t regionCount[TR_SEGS / 32];  // entries in each warp's region of pass
};

// order-preserving u32 image of a float (NaN excluded by the caller)
__device__ __forceinline__ uint32_t orderedBits(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float orderedFloat(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// view-space depth bin of a passing pixel (:196-203, getHairDepthBoundsVS :242-246)
__device__ __forceinline__ uint32_t viewDepthBin(const HfbUniforms& U, uint32_t B, float dv0, float dv1, f2 p,
                                                 float hd) {
  const f3 vs = projectVertex(U.projMatrixInv.m, mk4(p.x, p.y, hd, 1.0f));
  return (B - 1u) - getDepthBin(B, dv0, dv1, vs.z);
}

// A (segment, tile) record keeps the smallest bin over its passing pixels.
// When the inverse projection's z row is (0, 0, m10, m14) and its w row
// (0, 0, m11, m15) -- a perspective or orthographic projection -- a pixel's
// view depth does not depend on the pixel: for x, y >= 0 the zero entries
// give signed zeros that the sums absorb, so z = m14 / RN(RN(m11 h) + m15)
// when |m10 h| stays below a quarter ulp of m14 (the z row then rounds to
// m14 exactly).  That is a monotone function of the depth h while the
// denominator keeps one sign, and getDepthBin is monotone in z (u32(NaN)
// is 0), so the smallest bin over a set of depths is the bin of its smallest
// or of its largest depth: the record needs two bins, not one per pixel.
// binRange returns the range [lo, hi] of depths over which that holds for a
// segment (empty when it does not): its four projected depths widened by
// 1e-5 of their magnitude -- the interpolated depths, mixes of the four with
// weights clamped to [0, 1], stay within 1e-6 of it -- checked on both ends.
__device__ __forceinline__ bool binRowsFromDepth(const float* M) {
  return (__float_as_uint(M[2]) << 1) == 0u && (__float_as_uint(M[6]) << 1) == 0u &&
         (__float_as_uint(M[3]) << 1) == 0u && (__float_as_uint(M[7]) << 1) == 0u && M[14] != 0.0f &&
         M[15] != 0.0f && isfinite(M[10]) && isfinite(M[11]) && isfinite(M[14]) && isfinite(M[15]);
}

__device__ __forceinline__ void binRange(const float* M, bool rows, f4 dp, float& lo, float& hi) {
  lo = __int_as_float(0x7f800000);
  hi = -lo;
  if (!rows) return;
  const float a = fminf(fminf(dp.x, dp.y), fminf(dp.z, dp.w)), b = fmaxf(fmaxf(dp.x, dp.y), fmaxf(dp.z, dp.w));
  const bool finite = isfinite(dp.x) && isfinite(dp.y) && isfinite(dp.z) && isfinite(dp.w);
  if (!finite || !(fabsf(a) < 1e30f && fabsf(b) < 1e30f)) return;
  const float m = fadd(fmul(1e-5f, fadd(fabsf(a), fabsf(b))), 1e-30f);
  const float l = fsub(a, m), h = fadd(b, m);
  if (!(fmul(fmul(fabsf(M[10]), fmaxf(fabsf(l), fabsf(h))), 1.0001f) < fmul(fabsf(M[14]), 0x1p-26f))) return;
  const float w0 = fadd(fmul(M[11], l), M[15]), w1 = fadd(fmul(M[11], h), M[15]);
  if (isfinite(w0) && isfinite(w1) && ((w0 > 0.0f && w1 > 0.0f) || (w0 < 0.0f && w1 < 0.0f))) {
    lo = l;
    hi = h;
  }
}

// Stores one (segment, tile) record, :220-237 (warp-aggregated pointer
// allocation; min / max depth as u32 maxima, order independent).
__device__ __forceinline__ void storeTileRecord(uint4* __restrict__ tiles, uint32_t* __restrict__ segBuf,
                                               uint32_t* __restrict__ segCount, uint32_t* __restrict__ binCount,
                                               DeviceCounters* __restrict__ counters, uint32_t maxDrawn,
                                               uint32_t tilesX, uint32_t B, uint32_t tx, uint32_t ty,
                                               uint32_t dbin, float dmin, float dmax, uint32_t key, uint32_t T) {
  if (!HFB_EXPECT(tx < tilesX && ty * tilesX + tx < T && dbin < B)) return;
  cg::coalesced_group g = cg::coalesced_threads();
  uint32_t base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(HFB_G(&segBuf[0]), g.size());
  base = g.shfl(base, 0);
  const uint32_t ptr = base + g.thread_rank();
  if (ptr < maxDrawn) {
    const uint32_t ti = ty * tilesX * B + tx * B + dbin;
    atomicMax(HFB_G(&tiles[ti].x), f2u(fmul(fsub(1.0f, dmin), F_MAX_U32)));  // _storeTileHead
    atomicMax(HFB_G(&tiles[ti].y), f2u(fmul(dmax, F_MAX_U32)));
    atomicAdd(HFB_G(&segCount[ty * tilesX + tx]), 1u);  // _incTileSegmentCount
    atomicAdd(HFB_G(&binCount[ti]), 1u);
    // staging record in the list slot; binFinalize rewrites it
    (*HFB_G(&segBuf[1u + 2u * ptr])) = ti;
    (*HFB_G(&segBuf[2u + 2u * ptr])) = key;
  } else {
    atomicAdd(HFB_G(&counters->tileRecordsDropped), 1ull);
  }
}

// processTile for every tile of one segment's tile range, by one thread.
__device__ void rasterSegmentSerial(const HfbUniforms& U, const ProjSeg& s, uint32_t W, uint32_t H, uint32_t TS,
                                    uint32_t B, uint32_t tilesX, uint32_t maxDrawn, float dv0, float dv1,
                                    uint32_t key, uint32_t ux0, uint32_t uy0, uint32_t ux1, uint32_t uy1,
                                    const float* __restrict__ depth, uint4* __restrict__ tiles,
                                    uint32_t* __restrict__ segBuf, uint32_t* __restrict__ segCount,
                                    uint32_t* __restrict__ binCount, DeviceCounters* __restrict__ counters) {
  const uint32_t tminx = ux0 / TS, tminy = uy0 / TS, tmaxx = ux1 / TS, tmaxy = uy1 / TS;
  const RowSpan span = makeRowSpan(s);
  for (uint32_t ty = tminy; ty <= tmaxy; ty++) {
    for (uint32_t tx = tminx; tx <= tmaxx; tx++) {
      TileB tb = tileBoundsPx(W, H, TS, tx, ty);
      // Only pixel corners inside the segment's bounding rectangle can pass
      // the four edge tests, so the walk is restricted to tile x rect, and
      // per row to the candidate span around the covered interval.
      const uint32_t xa = max(tb.x0, ux0), xb = min(tb.x1, ux1 + 1u);
      const uint32_t ya = max(tb.y0, uy0), yb = min(tb.y1, uy1 + 1u);
      float dmin = 999.0f, dmax = -999.0f;
      uint32_t dbin = B;
      for (uint32_t y = ya; y < yb; y++) {
        uint32_t x0r = xa, x1r = xb;
        span.candidates((float)y, x0r, x1r);
        for (uint32_t x = x0r; x < x1r; x++) {
          f2 p = mk2((float)x, (float)y);
          if (!insideQuad(s, p)) continue;
          f2 w = interpolateHairQuad(s, p);
          float hd = interpolateHairF32(w, s.depthsProj);
          float zb = loadTex2DClamp(depth, W, H, (int)x, (int)H - (int)y);
          if (hd > zb) continue;  // depth test, :193-195
          dmin = fminf(dmin, hd);
          dmax = fmaxf(dmax, hd);
          dbin = min(dbin, viewDepthBin(U, B, dv0, dv1, p, hd));
        }
      }
      if (dmin > 1.0f) continue;
      storeTileRecord(tiles, segBuf, segCount, binCount, counters, maxDrawn, tilesX, B, tx, ty, dbin, dmin, dmax,
                      key, tilesX * divCeil(H, TS));
    }
  }
}

template <uint32_t TR_SLOTS, uint32_t TR_CHUNK>
__device__ __forceinline__ void tilesRasterBody(const HfbUniforms& U, uint32_t P, uint32_t nStrands, uint32_t TS,
                                                uint32_t B, uint32_t threshold, float4 bsphere,
                                                const float4* __restrict__ pos, const float4* __restrict__ tan,
                                                const float* __restrict__ depth, uint4* __restrict__ tiles,
                                                uint32_t* __restrict__ segBuf, uint32_t* __restrict__ segCount,
                                                uint32_t* __restrict__ binCount,
                                                DeviceCounters* __restrict__ counters, TrShared<TR_SLOTS, TR_CHUNK>& sh,
                                                uint32_t blk, float4* __restrict__ projOut) {
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  const uint32_t segsPerStrand = P - 1u;
  const uint32_t nSeg = nStrands * segsPerStrand;
  const uint32_t gid = blk * TR_SEGS + tid;
  const f2 size = mk2(U.viewport.x, U.viewport.y);
  const uint32_t W = f2u(size.x), H = f2u(size.y);
  const uint32_t tilesX = divCeil(W, TS);
  const uint32_t maxDrawn = U.maxDrawnHairSegments;
  // getHairDepthBoundsVS, :242-246
  const f4 bsVS = m4v(U.modelViewMat.m, mk4(bsphere.x, bsphere.y, bsphere.z, 1.0f));
  const float dv0 = fsub(bsVS.z, bsphere.w), dv1 = fadd(bsVS.z, bsphere.w);
  const bool binRows = binRowsFromDepth(U.projMatrixInv.m);
  const uint32_t tsShift = (uint32_t)(__ffs((int)TS) - 1);  // TS is 8, 16 or 32

  // ---- project this thread's segment ----
  uint32_t pairs = 0, slots = 0, key = 0;
  bool serial = false;
  ProjSeg s;
  uint32_t ux0 = 0, uy0 = 0, ux1 = 0, uy1 = 0;
  if (gid < nSeg) {
    const uint32_t strand = gid / segsPerStrand, seg = gid - strand * segsPerStrand;
    key = (strand << 8) | seg;
    s = projectSegment(U, pos, tan, P, strand, seg, size);
    if (projOut) {  // for the fine pass of the same frame
      float4* o = projOut + (size_t)gid * SEG_PROJ_VEC4;
      o[0] = make_float4(s.v00.x, s.v00.y, s.v01.x, s.v01.y);
      o[1] = make_float4(s.v10.x, s.v10.y, s.v11.x, s.v11.y);
      o[2] = make_float4(s.depthsProj.x, s.depthsProj.y, s.depthsProj.z, s.depthsProj.w);
    }
    // getRasterizedHairBounds, swRasterizeHair.wgsl.ts:111-124
    const float bx1 = fminf(ceilf(fmaxf(fmaxf(s.v00.x, s.v01.x), fmaxf(s.v10.x, s.v11.x))), size.x);
    const float by1 = fminf(ceilf(fmaxf(fmaxf(s.v00.y, s.v01.y), fmaxf(s.v10.y, s.v11.y))), size.y);
    const float bx0 = fmaxf(floorf(fminf(fminf(s.v00.x, s.v01.x), fminf(s.v10.x, s.v11.x))), 0.0f);
    const float by0 = fmaxf(floorf(fminf(fminf(s.v00.y, s.v01.y), fminf(s.v10.y, s.v11.y))), 0.0f);
    ux0 = f2u(bx0); uy0 = f2u(by0); ux1 = f2u(bx1); uy1 = f2u(by1);
    const uint32_t tminx = ux0 / TS, tminy = uy0 / TS, tmaxx = ux1 / TS, tmaxy = uy1 / TS;
    const uint32_t tsx = (tmaxx - tminx) + 1u, tsy = (tmaxy - tminy) + 1u;
    if (tsx * tsy <= threshold) {  // degenerate segment rejection, :111-117
      const uint32_t cx1 = min(ux1 + 1u, W - 1u), cy1 = min(uy1 + 1u, H - 1u);
      const uint32_t cwid = cx1 > ux0 ? cx1 - ux0 : 0u, chei = cy1 > uy0 ? cy1 - uy0 : 0u;
      if (cwid && chei) {
        if ((uint64_t)cwid * chei >= (1ull << 24) || cwid > 4096u || chei > 8192u) {
          serial = true;  // beyond the pair encoding: its own walk
        } else {
          pairs = cwid * chei;
          slots = tsx * tsy;
        }
      }
      sh.cx0[tid] = ux0; sh.cy0[tid] = uy0; sh.cw[tid] = max(cwid, 1u);
      sh.tminx[tid] = tminx; sh.tminy[tid] = tminy; sh.tsx[tid] = tsx;
      const f2 o[4] = {s.v01, s.v11, s.v10, s.v00};  // the edge tests in insideQuad's order
      const f2 e[4] = {s.v00, s.v01, s.v11, s.v10};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        sh.ox[i][tid] = o[i].x;
        sh.oy[i][tid] = o[i].y;
        sh.ex[i][tid] = fsub(e[i].x, o[i].x);
        sh.ey[i][tid] = fsub(e[i].y, o[i].y);
      }
      sh.dp[0][tid] = s.depthsProj.x; sh.dp[1][tid] = s.depthsProj.y;
      sh.dp[2][tid] = s.depthsProj.z; sh.dp[3][tid] = s.depthsProj.w;
      float blo, bhi;
      binRange(U.projMatrixInv.m, binRows, s.depthsProj, blo, bhi);
      sh.blo[tid] = blo; sh.bhi[tid] = bhi;
      const QuadConst q = quadConst(s);
      sh.qsx[tid] = q.sm.x; sh.qsy[tid] = q.sm.y; sh.qax[tid] = q.ab.x; sh.qay[tid] = q.ab.y;
      sh.qd2[tid] = q.d2; sh.qlse[tid] = q.lse; sh.qws[tid] = q.wS; sh.qwe[tid] = q.wE; sh.qd22[tid] = q.d22;
    }
  }
  // accumulators of the block's (segment, tile) pairs; segments beyond them walk alone
  uint32_t slotTotal;
  const uint32_t slotEx = blockExclusiveScan(slots, sh.warpSums, slotTotal);
  if (slots && slotEx + slots > TR_SLOTS) {
    serial = true;
    pairs = 0;
    slots = 0;
  }
  sh.slotBase[tid] = slotEx;
  uint32_t pairTotal;
  sh.pairBase[tid] = blockExclusiveScan(pairs, sh.warpSums, pairTotal);
  if (tid == 0) sh.pairBase[TR_SEGS] = pairTotal;
  for (uint32_t i = tid; i < TR_SLOTS; i += TR_SEGS) {
    sh.accMin[i] = 0xffffffffu;
    sh.accMax[i] = 0u;
    sh.accBin[i] = B;
  }
  __syncthreads();

  // Each thread walks one contiguous range of the block's pairs.  A round's
  // A1 appends passing pairs to its warp's region of the list (a count kept
  // in registers: no atomic) until a region is full; the warp then stops,
  // its lanes at the pairs they have not yet appended, which the next round
  // retests.  A2 then has a full list to share out, and the block meets at
  // its barriers about once per TR_CHUNK passing pixels rather than once per
  // TR_CHUNK candidate pairs.
  // edgeFunction (swRasterizeHair.wgsl.ts:128-130) is (x - ox) * ey - (y - oy) * ex: the
  // second product is the same along a row and is formed once per row (the same values)
  constexpr uint32_t REGION = TR_CHUNK / (TR_SEGS / 32);
  const uint32_t warp = tid >> 5;
  const uint32_t per = divCeil(pairTotal, TR_SEGS);
  uint32_t p = tid * per;
  const uint32_t pEnd = min(p + per, pairTotal);
  uint32_t k = 0, rx = 0, ry = 0, w = 1, x0 = 0, y0 = 0;
  float eox[4], eey[4], rowT[4];
  auto loadSeg = [&](uint32_t kk) {
    x0 = sh.cx0[kk]; y0 = sh.cy0[kk]; w = sh.cw[kk];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      eox[i] = sh.ox[i][kk]; eey[i] = sh.ey[i][kk];
    }
  };
  auto setRow = [&]() {
    const float py = (float)(y0 + ry);
#pragma unroll
    for (int i = 0; i < 4; i++) rowT[i] = fmul(fsub(py, sh.oy[i][k]), sh.ex[i][k]);
  };
  if (p < pEnd) {
    uint32_t lo = 0, hi = TR_SEGS;  // last k with pairBase[k] <= p
    while (hi - lo > 1u) {
      const uint32_t mid = (lo + hi) >> 1;
      if (sh.pairBase[mid] <= p) lo = mid; else hi = mid;
    }
    k = lo;
    loadSeg(k);
    const uint32_t r = p - sh.pairBase[k];
    ry = r / w;
    rx = r - ry * w;
    setRow();
  }
  while (__syncthreads_or(p < pEnd)) {
    // ---- A1: edge tests along the thread's range until the warp's region is full ----
    uint32_t* const region = sh.pass + warp * REGION;
    uint32_t cnt = 0;  // the warp's entries (the same in every lane)
    while (cnt < REGION) {
      const bool act = p < pEnd;
      if (!__any_sync(0xffffffffu, act)) break;
      bool pass = false;
      if (act) {
        const float px = (float)(x0 + rx);
        pass = true;
#pragma unroll
        for (int i = 0; i < 4; i++) {  // edgeFunction >= 0
          const float C = fsub(fmul(fsub(px, eox[i]), eey[i]), rowT[i]);
          pass = pass && C >= 0.0f;
        }
      }
      const uint32_t bal = __ballot_sync(0xffffffffu, pass);
      const uint32_t at = cnt + __popc(bal & ((1u << lane) - 1u));
      const bool fits = !pass || at < REGION;  // else the region is full: the pair goes first next round
      if (pass && fits && HFB_EXPECT(k < TR_SEGS)) region[at] = k | (rx << 7) | (ry << 19);
      cnt = min(cnt + (uint32_t)__popc(bal), REGION);
      if (act && fits) {
        p++;
        if (++rx == w) {
          rx = 0;
          ry++;
          if (p < pEnd && p >= sh.pairBase[k + 1u]) {  // next segment with pairs
            while (sh.pairBase[k + 1u] <= p) k++;
            loadSeg(k);
            ry = 0;
          }
          if (p < pEnd) setRow();
        }
      }
    }
    if (lane == 0) sh.regionCount[warp] = cnt;
    __syncthreads();
    // ---- A2: depth, depth test and bin of every passing pixel ----
    uint32_t rc[TR_SEGS / 32], nPass = 0;
#pragma unroll
    for (uint32_t r = 0; r < TR_SEGS / 32; r++) {
      rc[r] = sh.regionCount[r];
      nPass += rc[r];
    }
    for (uint32_t i = tid; i < nPass; i += TR_SEGS) {
      uint32_t r = 0, o = i;  // entry i of the regions laid end to end
#pragma unroll
      for (uint32_t q = 0; q + 1u < TR_SEGS / 32; q++)
        if (r == q && o >= rc[q]) { o -= rc[q]; r++; }
      const uint32_t e = sh.pass[r * REGION + o];
      const uint32_t k = e & 0x7fu, rx = (e >> 7) & 0xfffu, ry = e >> 19;
      const uint32_t x = sh.cx0[k] + rx, y = sh.cy0[k] + ry;
      const f2 p = mk2((float)x, (float)y);
      QuadConst qc;
      qc.sm = mk2(sh.qsx[k], sh.qsy[k]);
      qc.ab = mk2(sh.qax[k], sh.qay[k]);
      qc.d2 = sh.qd2[k]; qc.lse = sh.qlse[k]; qc.wS = sh.qws[k]; qc.wE = sh.qwe[k];
      qc.ab2 = mk2(sh.ex[3][k], sh.ey[3][k]);
      qc.d22 = sh.qd22[k];
      const f2 wq = interpolateHairQuadPre(qc, mk2(sh.ox[3][k], sh.oy[3][k]), p);
      const float hd = interpolateHairF32(wq, mk4(sh.dp[0][k], sh.dp[1][k], sh.dp[2][k], sh.dp[3][k]));
      const float zb = loadTex2DClamp(depth, W, H, (int)x, (int)H - (int)y);
      if (hd > zb) continue;  // depth test, :193-195
      const uint32_t slot =
          sh.slotBase[k] + ((y >> tsShift) - sh.tminy[k]) * sh.tsx[k] + ((x >> tsShift) - sh.tminx[k]);
      if (!HFB_EXPECT(slot < TR_SLOTS)) continue;
      if (!(hd >= sh.blo[k] && hd <= sh.bhi[k]))  // else the record's bin comes from its depth range (E)
        atomicMin(&sh.accBin[slot], viewDepthBin(U, B, dv0, dv1, p, hd));
      if (!isnan(hd)) {  // fminf / fmaxf ignore a NaN depth
        atomicMin(&sh.accMin[slot], orderedBits(hd));
        atomicMax(&sh.accMax[slot], orderedBits(hd));
      }
    }
  }  // the loop's barrier ends A2 before the next round and before E

  // ---- E: one record per (segment, tile) that took a pixel ----
  for (uint32_t i = tid; i < slotTotal && i < TR_SLOTS; i += TR_SEGS) {
    if (sh.accMin[i] == 0xffffffffu) continue;  // no pixel with a depth
    const float dmin = orderedFloat(sh.accMin[i]);
    if (dmin > 1.0f) continue;
    uint32_t lo = 0, hi = TR_SEGS;  // segment of the slot: last k with slotBase[k] <= i
    while (hi - lo > 1u) {
      const uint32_t mid = (lo + hi) >> 1;
      if (sh.slotBase[mid] <= i) lo = mid; else hi = mid;
    }
    const uint32_t k = lo, l = i - sh.slotBase[k];
    const uint32_t ty = sh.tminy[k] + l / sh.tsx[k], tx = sh.tminx[k] + l % sh.tsx[k];
    const uint32_t g = blk * TR_SEGS + k;
    const uint32_t strand = g / segsPerStrand, seg = g - strand * segsPerStrand;
    const float dmax = orderedFloat(sh.accMax[i]);
    uint32_t bin = sh.accBin[i];
    if (sh.blo[k] <= sh.bhi[k]) {  // the smallest bin is at one end of the depths (binRange)
      const f2 p0 = mk2(0.0f, 0.0f);
      bin = min(bin, min(viewDepthBin(U, B, dv0, dv1, p0, dmin), viewDepthBin(U, B, dv0, dv1, p0, dmax)));
    }
    storeTileRecord(tiles, segBuf, segCount, binCount, counters, maxDrawn, tilesX, B, tx, ty, bin, dmin, dmax,
                    (strand << 8) | seg, tilesX * divCeil(H, TS));
  }
  if (serial)
    rasterSegmentSerial(U, s, W, H, TS, B, tilesX, maxDrawn, dv0, dv1, key, ux0, uy0, ux1, uy1, depth, tiles,
                        segBuf, segCount, binCount, counters);
  __syncthreads();  // the block's staging is reused by its next segments
}

__global__ void __launch_bounds__(TR_SEGS, 6)
tilesRasterKernel(const HfbUniforms U, uint32_t P, uint32_t nStrands, uint32_t TS, uint32_t B,
                  uint32_t threshold, float4 bsphere, const float4* __restrict__ pos,
                  const float4* __restrict__ tan, const float* __restrict__ depth, uint4* __restrict__ tiles,
                  uint32_t* __restrict__ segBuf, uint32_t* __restrict__ segCount,
                  uint32_t* __restrict__ binCount, DeviceCounters* __restrict__ counters, float4* __restrict__ proj) {
  __shared__ TrShared<TR_SLOTS, TR_CHUNK> sh;
  tilesRasterBody<TR_SLOTS, TR_CHUNK>(U, P, nStrands, TS, B, threshold, bsphere, pos, tan, depth, tiles, segBuf,
                                      segCount, binCount, counters, sh, blockIdx.x, proj);
}

// ---------------------------------------------------------------------------
// 2. binScan: exclusive prefix over T*B counts (block-local + block sums)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void binScanBlocksBody(const uint32_t* __restrict__ cnt, uint32_t* __restrict__ off,
                                                  uint32_t* __restrict__ blockSums, uint32_t n, uint32_t* warpSums,
                                                  uint32_t blk) {
  const uint32_t base = blk * SCAN_PER_BLOCK + threadIdx.x * 4u;
  uint32_t v[4], s = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[k] = base + k < n ? (*HFB_G(&cnt[base + k])) : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t ex = blockExclusiveScan(s, warpSums, total);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (base + k < n) (*HFB_G(&off[base + k])) = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0) (*HFB_G(&blockSums[blk])) = total;
}

__global__ void __launch_bounds__(512) binScanBlocks(const uint32_t* __restrict__ cnt, uint32_t* __restrict__ off,
                                                     uint32_t* __restrict__ blockSums, uint32_t n) {
  __shared__ uint32_t warpSums[32];
  binScanBlocksBody(cnt, off, blockSums, n, warpSums, blockIdx.x);
}

__device__ __forceinline__ void binScanSumsBody(uint32_t* __restrict__ blockSums, uint32_t nBlocks,
                                                uint32_t* warpSums) {
  uint32_t carry = 0;
  for (uint32_t b0 = 0; b0 < nBlocks; b0 += blockDim.x) {
    uint32_t i = b0 + threadIdx.x;
    uint32_t v = i < nBlocks ? (*HFB_G(&blockSums[i])) : 0u;
    uint32_t total;
    uint32_t ex = blockExclusiveScan(v, warpSums, total);
    if (i < nBlocks) (*HFB_G(&blockSums[i])) = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(1024) binScanSums(uint32_t* __restrict__ blockSums, uint32_t nBlocks) {
  __shared__ uint32_t warpSums[32];
  binScanSumsBody(blockSums, nBlocks, warpSums);
}

// ---------------------------------------------------------------------------
// 3. binScatter: keys into CSR order (order inside a bin fixed by step 4)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void binScatterBody(const uint32_t* __restrict__ segBuf, uint32_t maxDrawn,
                                               uint32_t* __restrict__ binOffset,
                                               const uint32_t* __restrict__ blockSums, uint32_t* __restrict__ keys,
                                               DeviceCounters* __restrict__ counters, uint32_t blk, uint32_t nblk,
                                               uint32_t TB) {
  const uint32_t total = (*HFB_G(&segBuf[0]));
  const uint32_t n = min(total, maxDrawn);
  if (blk == 0 && threadIdx.x == 0) atomicAdd(HFB_G(&counters->tileRecords), (unsigned long long)total);
  for (uint32_t r = blk * blockDim.x + threadIdx.x; r < n; r += nblk * blockDim.x) {
    uint32_t ti = (*HFB_G(&segBuf[1u + 2u * r]));
    uint32_t key = (*HFB_G(&segBuf[2u + 2u * r]));
    if (!HFB_EXPECT(ti < TB)) continue;
    uint32_t pos = (*HFB_G(&blockSums[ti / SCAN_PER_BLOCK])) + atomicAdd(HFB_G(&binOffset[ti]), 1u);
    if (HFB_EXPECT(pos < maxDrawn)) (*HFB_G(&keys[pos])) = key;
  }
}

__global__ void __launch_bounds__(256)
binScatterKernel(const uint32_t* __restrict__ segBuf, uint32_t maxDrawn, uint32_t* __restrict__ binOffset,
                 const uint32_t* __restrict__ blockSums, uint32_t* __restrict__ keys,
                 DeviceCounters* __restrict__ counters, uint32_t TB) {
  binScatterBody(segBuf, maxDrawn, binOffset, blockSums, keys, counters, blockIdx.x, gridDim.x, TB);
}

// ---------------------------------------------------------------------------
// 4. binFinalize: per-bin sort + reference linked list (warp per bin)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void writeList(uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles, uint32_t ti,
                                          uint32_t start, uint32_t i, uint32_t n, uint32_t key) {
  // _storeTileSegment encoding: (segment << 24) | strand; next = previous
  // (smaller) key, so the walk from the head visits keys in descending order.
  uint32_t p = start + i;
  (*HFB_G(&segBuf[1u + 2u * p])) = ((key & 0xffu) << 24) | (key >> 8);
  (*HFB_G(&segBuf[2u + 2u * p])) = i == 0 ? INVALID_PTR : p - 1u;
  if (i == n - 1u) {
    (*HFB_G(&tiles[ti])).z = p + 1u;  // head pointer (+1, 0 = empty)
    (*HFB_G(&tiles[ti])).w = n;       // padding0: list length, a hint the fine pass verifies
  }
}

// Bitonic sorting network (Batcher) on N keys in shared memory, ascending, N a
// power of two >= 64.  Stage (k, j) compares the keys at x and x + j for every
// x with bit j clear, ascending where bit k of x is clear.  The stages with
// j <= 32 stay inside aligned runs of 64 keys: a warp holds such a run in
// registers (positions p and p + 32 in lane p % 32; the j = 32 exchange within
// a lane, j <= 16 across lanes by shuffles) and runs all of them between two
// passes over shared memory.

// The j <= 32 stages of the merge steps k = kFrom .. kTo (doubling) on every
// 64-key run; the caller's warps warp0, warp0 + nWarps, ... take the runs.
__device__ __forceinline__ void bitonicRuns64(uint32_t* s, uint32_t N, uint32_t kFrom, uint32_t kTo, uint32_t lane,
                                              uint32_t warp0, uint32_t nWarps) {
  for (uint32_t r = warp0; r < N / 64u; r += nWarps) {
    const uint32_t p0 = r * 64u + lane, p1 = p0 + 32u;
    uint32_t e0 = s[p0], e1 = s[p1];
    for (uint32_t k = kFrom; k <= kTo; k <<= 1) {
      uint32_t j = k >> 1;
      if (j >= 32u) {
        const bool asc = (p0 & k) == 0u;
        const uint32_t lo = min(e0, e1), hi = max(e0, e1);
        e0 = asc ? lo : hi;
        e1 = asc ? hi : lo;
        j = 16u;
      }
      for (; j > 0u; j >>= 1) {
        const uint32_t o0 = __shfl_xor_sync(0xffffffffu, e0, j), o1 = __shfl_xor_sync(0xffffffffu, e1, j);
        const bool low = (lane & j) == 0u;
        e0 = (((p0 & k) == 0u) == low) ? min(e0, o0) : max(e0, o0);
        e1 = (((p1 & k) == 0u) == low) ? min(e1, o1) : max(e1, o1);
      }
    }
    s[p0] = e0;
    s[p1] = e1;
  }
}

// Sorts s[0, N).  BLOCK: every thread of the block calls it (block barriers);
// else one warp does (warp barriers).
template <bool BLOCK>
__device__ __forceinline__ void bitonicSort(uint32_t* s, uint32_t N) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t t0 = BLOCK ? threadIdx.x : lane, nT = BLOCK ? blockDim.x : 32u;
  const uint32_t w0 = BLOCK ? threadIdx.x >> 5 : 0u, nW = BLOCK ? blockDim.x >> 5 : 1u;
  auto sync = [] { if (BLOCK) __syncthreads(); else __syncwarp(); };
  bitonicRuns64(s, N, 2u, 64u, lane, w0, nW);
  sync();
  for (uint32_t k = 128u; k <= N; k <<= 1) {
    for (uint32_t j = k >> 1; j >= 64u; j >>= 1) {
      const uint32_t lj = __ffs(j) - 1u;  // j = 2^lj
      for (uint32_t c = t0; c < N / 2u; c += nT) {
        const uint32_t a = ((c >> lj) << (lj + 1u)) | (c & (j - 1u)), b = a + j;
        const uint32_t x = s[a], y = s[b];
        if ((x > y) == ((a & k) == 0u)) { s[a] = y; s[b] = x; }
      }
      sync();
    }
    bitonicRuns64(s, N, k, k, lane, w0, nW);
    sync();
  }
}

// Sorts and links the larger bin ti (more than 8 records) with the whole warp.
__device__ __forceinline__ void finalizeBinWarp(uint32_t ti, uint32_t n, uint32_t start, uint32_t lane,
                                                uint32_t* __restrict__ keys, uint32_t* __restrict__ segBuf,
                                                uint4* __restrict__ tiles, uint32_t* __restrict__ largeBins,
                                                uint32_t* s) {
  if (n <= SMALL_BIN) {
    uint32_t v = lane < n ? (*HFB_G(&keys[start + lane])) : 0xffffffffu;
    // bitonic sort across the warp, ascending
#pragma unroll
    for (uint32_t k = 2; k <= 32; k <<= 1) {
#pragma unroll
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        uint32_t o = __shfl_xor_sync(0xffffffffu, v, j);
        bool asc = (lane & k) == 0, low = (lane & j) == 0;
        v = (asc == low) ? min(v, o) : max(v, o);
      }
    }
    if (lane < n) writeList(segBuf, tiles, ti, start, lane, n, v);
  } else if (n <= MEDIUM_BIN) {
    uint32_t N = 64;
    while (N < n) N <<= 1;
    for (uint32_t i = lane; i < N; i += 32) s[i] = i < n ? (*HFB_G(&keys[start + i])) : 0xffffffffu;
    __syncwarp();
    bitonicSort<false>(s, N);
    for (uint32_t i = lane; i < n; i += 32) writeList(segBuf, tiles, ti, start, i, n, s[i]);
    __syncwarp();
  } else if (lane == 0) {
    uint32_t slot = atomicAdd(HFB_G(&largeBins[0]), 1u);
    (*HFB_G(&largeBins[1u + slot])) = ti;
  }
}

// One warp per bin, the warps of the grid striding over the bins (the
// single-instance launch: a fixed grid, where spreading the larger bins over
// every warp keeps the tail short).
__device__ __forceinline__ void binFinalizeWarpBody(uint32_t TB, const uint32_t* __restrict__ binCount,
                                                    const uint32_t* __restrict__ binOffset,
                                                    const uint32_t* __restrict__ blockSums,
                                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ segBuf,
                                                    uint4* __restrict__ tiles, uint32_t* __restrict__ largeBins,
                                                    uint32_t (*smem)[MEDIUM_BIN], uint32_t blk, uint32_t nblk) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t gw = (blk * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (nblk * blockDim.x) >> 5;
  const uint32_t drawn = (*HFB_G(&segBuf[0]));
  for (uint32_t ti = gw; ti < TB; ti += nw) {
    const uint32_t n = (*HFB_G(&binCount[ti]));
    if (n == 0) continue;
    const uint32_t end = (*HFB_G(&blockSums[ti / SCAN_PER_BLOCK])) + (*HFB_G(&binOffset[ti]));  // bin end
    if (!HFB_EXPECT(n <= end && end <= drawn)) continue;
    finalizeBinWarp(ti, n, end - n, lane, keys, segBuf, tiles, largeBins, smem[warp]);
  }
}

// A block takes 32 consecutive bins at a time (blockDim 256: 8 warps of 4
// bins): a group of 8 lanes sorts and links a bin of at most 8 records (most
// bins), the larger ones go to a block queue that the warps then share, one
// warp per bin.  All threads of the block call it.  (The batched launch,
// whose persistent blocks take these 32-bin pieces dynamically.)
__device__ __forceinline__ void binFinalizeBody(uint32_t TB, const uint32_t* __restrict__ binCount,
                                                const uint32_t* __restrict__ binOffset,
                                                const uint32_t* __restrict__ blockSums, uint32_t* __restrict__ keys,
                                                uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles,
                                                uint32_t* __restrict__ largeBins, uint32_t (*smem)[MEDIUM_BIN],
                                                uint32_t blk, uint32_t nblk) {
  __shared__ uint32_t bigTi[32], bigN[32], bigEnd[32], nBig;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nWarps = blockDim.x >> 5;
  const uint32_t grp = lane >> 3, gl = lane & 7u;  // four groups of 8 lanes
  const uint32_t perBlock = nWarps * 4u;
  const uint32_t drawn = (*HFB_G(&segBuf[0]));
  uint32_t* s = smem[warp];
  for (uint32_t bbase = blk * perBlock; bbase < TB; bbase += nblk * perBlock) {
    if (threadIdx.x == 0) nBig = 0;
    __syncthreads();
    const uint32_t tg = bbase + warp * 4u + grp;
    uint32_t ng = 0, endg = 0;
    if (tg < TB) {
      ng = (*HFB_G(&binCount[tg]));
      if (ng) endg = (*HFB_G(&blockSums[tg / SCAN_PER_BLOCK])) + (*HFB_G(&binOffset[tg]));  // bin end
    }
    const bool ok = ng != 0u && HFB_EXPECT(ng <= endg && endg <= drawn);
    const bool small = ok && ng <= 8u;
    const uint32_t smallLanes = __ballot_sync(0xffffffffu, small);
    if (small) {
      const uint32_t start = endg - ng;
      uint32_t v = gl < ng ? (*HFB_G(&keys[start + gl])) : 0xffffffffu;
      // bitonic sort across the group's 8 lanes, ascending
#pragma unroll
      for (uint32_t k = 2; k <= 8; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
          const uint32_t o = __shfl_xor_sync(smallLanes, v, j);
          const bool asc = (gl & k) == 0, low = (gl & j) == 0;
          v = (asc == low) ? min(v, o) : max(v, o);
        }
      }
      if (gl < ng) writeList(segBuf, tiles, tg, start, gl, ng, v);
    } else if (ok && gl == 0u) {
      const uint32_t q = atomicAdd(&nBig, 1u);  // < 32: one per group of the block
      bigTi[q] = tg;
      bigN[q] = ng;
      bigEnd[q] = endg;
    }
    __syncthreads();
    const uint32_t nb = nBig;
    for (uint32_t q = warp; q < nb; q += nWarps)
      finalizeBinWarp(bigTi[q], bigN[q], bigEnd[q] - bigN[q], lane, keys, segBuf, tiles, largeBins, s);
    __syncthreads();  // the queue is rewritten by the next 32 bins
  }
}

__global__ void __launch_bounds__(256)
binFinalizeKernel(uint32_t TB, const uint32_t* __restrict__ binCount, const uint32_t* __restrict__ binOffset,
                  const uint32_t* __restrict__ blockSums, uint32_t* __restrict__ keys,
                  uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles, uint32_t* __restrict__ largeBins) {
  __shared__ uint32_t smem[8][MEDIUM_BIN];
  binFinalizeWarpBody(TB, binCount, binOffset, blockSums, keys, segBuf, tiles, largeBins, smem, blockIdx.x,
                      gridDim.x);
}

// ---------------------------------------------------------------------------
// 5. largeBins: one CTA per bin with > MEDIUM_BIN records.  A bin of at most
//    LARGE_SMEM_KEYS records is bitonic-sorted in shared memory and linked
//    from there; a larger one in runs of LARGE_SMEM_KEYS, then merged pairwise
//    through the bin's own list slots (free until the final write) by rank
//    search (keys are unique).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void largeBinsBody(const uint32_t* __restrict__ largeBins,
                                              const uint32_t* __restrict__ binCount,
                                              const uint32_t* __restrict__ binOffset,
                                              const uint32_t* __restrict__ blockSums, uint32_t* __restrict__ keys,
                                              uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles, uint32_t* sk,
                                              uint32_t vblk, uint32_t nvblk) {
  const uint32_t nLarge = (*HFB_G(&largeBins[0]));
  for (uint32_t li = vblk; li < nLarge; li += nvblk) {
    const uint32_t ti = (*HFB_G(&largeBins[1u + li]));
    const uint32_t n = (*HFB_G(&binCount[ti]));
    const uint32_t start = (*HFB_G(&blockSums[ti / SCAN_PER_BLOCK])) + (*HFB_G(&binOffset[ti])) - n;
    if (!HFB_EXPECT(start + n <= (*HFB_G(&segBuf[0])) && n > MEDIUM_BIN)) continue;
    uint32_t* a = keys + start;
    uint32_t* tmp = segBuf + 1u + 2u * start;  // 2n free words
    // sort runs in shared memory
    for (uint32_t r0 = 0; r0 < n; r0 += LARGE_SMEM_KEYS) {
      uint32_t m = min(LARGE_SMEM_KEYS, n - r0);
      uint32_t N = 64;
      while (N < m) N <<= 1;
      for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) sk[i] = i < m ? (*HFB_G(&a[r0 + i])) : 0xffffffffu;
      __syncthreads();
      bitonicSort<true>(sk, N);
      if (m == n) break;  // one run: the list is written from shared memory below
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) (*HFB_G(&a[r0 + i])) = sk[i];
      __syncthreads();
    }
    if (n <= LARGE_SMEM_KEYS) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) writeList(segBuf, tiles, ti, start, i, n, sk[i]);
      __syncthreads();
      continue;
    }
    // merge passes (ping-pong between a and tmp)
    uint32_t* src = a;
    uint32_t* dst = tmp;
    for (uint32_t run = LARGE_SMEM_KEYS; run < n; run <<= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t blk = i / (2u * run);
        uint32_t l0 = blk * 2u * run, l1 = min(l0 + run, n), r1 = min(l0 + 2u * run, n);
        uint32_t v = (*HFB_G(&src[i]));
        bool left = i < l1;
        uint32_t o0 = left ? l1 : l0, o1 = left ? r1 : l1;  // the other run
        uint32_t lo = o0, hi = o1;                           // count of other < v
        while (lo < hi) {
          uint32_t mid = (lo + hi) >> 1;
          if ((*HFB_G(&src[mid])) < v) lo = mid + 1; else hi = mid;
        }
        uint32_t rankOther = lo - o0;
        uint32_t rankSelf = i - (left ? l0 : l1);
        (*HFB_G(&dst[l0 + rankSelf + rankOther])) = v;
      }
      __syncthreads();
      uint32_t* t = src; src = dst; dst = t;
    }
    if (src != a) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) (*HFB_G(&a[i])) = (*HFB_G(&src[i]));
      __syncthreads();
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) writeList(segBuf, tiles, ti, start, i, n, (*HFB_G(&a[i])));
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024)
largeBinsKernel(const uint32_t* __restrict__ largeBins, const uint32_t* __restrict__ binCount,
                const uint32_t* __restrict__ binOffset, const uint32_t* __restrict__ blockSums,
                uint32_t* __restrict__ keys, uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles) {
  extern __shared__ uint32_t sk[];
  largeBinsBody(largeBins, binCount, binOffset, blockSums, keys, segBuf, tiles, sk, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// HairTileSortPass (count-tiles + sort) in one CTA, stable inside a bucket.
// ---------------------------------------------------------------------------
constexpr uint32_t SORT_MAX_BUCKETS = 256;

struct SortShared {
  uint32_t hist[SORT_MAX_BUCKETS], offs[SORT_MAX_BUCKETS], run[SORT_MAX_BUCKETS];
  uint32_t wcnt[32][SORT_MAX_BUCKETS];
  uint32_t drawn;
};

__device__ __forceinline__ void tileSortBody(uint32_t T, uint32_t NB, uint32_t bucketSize,
                                             const uint32_t* __restrict__ segCount, uint32_t* __restrict__ buckets,
                                             uint32_t* __restrict__ tileList, SortShared& ss) {
  uint32_t* hist = ss.hist;
  uint32_t* offs = ss.offs;
  uint32_t* run = ss.run;
  uint32_t (*wcnt)[SORT_MAX_BUCKETS] = ss.wcnt;
  uint32_t& drawn = ss.drawn;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  for (uint32_t b = tid; b < NB; b += blockDim.x) { hist[b] = 0; run[b] = 0; }
  if (tid == 0) drawn = 0;
  __syncthreads();
  // count-tiles: calcTileSortBucket, hairTileSortPass.countTiles.wgsl.ts:37-40
  uint32_t local = 0;
  for (uint32_t t = tid; t < T; t += blockDim.x) {
    uint32_t c = (*HFB_G(&segCount[t]));
    if (c > 0u) {
      atomicAdd(&hist[clampu(c / bucketSize, 0u, NB - 1u)], 1u);
      local++;
    }
  }
  atomicAdd(&drawn, local);
  __syncthreads();
  // calculateOffsetsForEachBucket: reverse exclusive scan, sort.wgsl.ts:68-75
  if (tid == 0) {
    uint32_t off = 0;
    for (uint32_t i = 0; i < NB; i++) {
      uint32_t idx = NB - 1u - i;
      offs[idx] = off;
      off += hist[idx];
    }
  }
  for (uint32_t b = tid; b < NB; b += blockDim.x) {
    (*HFB_G(&buckets[2u * b])) = hist[b];
    (*HFB_G(&buckets[2u * b + 1u])) = hist[b];  // the in-bucket write counter ends at tileCount
  }
  if (tid == 0) (*HFB_G(&tileList[0])) = drawn;
  __syncthreads();
  // stable scatter, one 1024-tile chunk at a time
  for (uint32_t c0 = 0; c0 < T; c0 += blockDim.x) {
    for (uint32_t i = tid; i < 32u * NB; i += blockDim.x) wcnt[i / NB][i % NB] = 0;
    __syncthreads();
    uint32_t t = c0 + tid;
    uint32_t c = t < T ? (*HFB_G(&segCount[t])) : 0u;
    bool valid = c > 0u;
    uint32_t b = valid ? clampu(c / bucketSize, 0u, NB - 1u) : SORT_MAX_BUCKETS;
    uint32_t peers = __match_any_sync(0xffffffffu, b);
    uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wcnt[warp][b] = __popc(peers);
    __syncthreads();
    for (uint32_t bb = tid; bb < NB; bb += blockDim.x) {
      uint32_t s = run[bb];
      for (uint32_t w = 0; w < 32; w++) {
        uint32_t x = wcnt[w][bb];
        wcnt[w][bb] = s;
        s += x;
      }
      run[bb] = s;
    }
    __syncthreads();
    if (valid && HFB_EXPECT(offs[b] + wcnt[warp][b] + rank < T)) (*HFB_G(&tileList[1u + offs[b] + wcnt[warp][b] + rank])) = t;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024)
tileSortKernel(uint32_t T, uint32_t NB, uint32_t bucketSize, const uint32_t* __restrict__ segCount,
               uint32_t* __restrict__ buckets, uint32_t* __restrict__ tileList) {
  __shared__ SortShared ss;
  tileSortBody(T, NB, bucketSize, segCount, buckets, tileList, ss);
}

// ---------------------------------------------------------------------------
// HairFinePass: persistent CTAs of TS x TS threads, one tile at a time.
//
// The tile's depth bins are processed in order (processTile per bin,
// hairFinePass.wgsl.ts:205-288).  Their lists are staged in rounds of up to
// STAGE segments -- short bins share a round, a long bin spans several -- and
// each round runs in three phases:
//   A1  one thread per (segment, row of the segment's tile-local bounding
//       box): the four edge tests of processHairSegment (:5-20) on every
//       pixel of the row into a bit mask; the passing pixels that are not
//       done are appended to a list, one shared atomic per warp;
//   A2  one thread per passing pair: segment-space interpolation, the depth
//       test and the fragment colour (:21-53), rounded through f16 like
//       pack2x16float (hairSlicesDataBuffer.ts:50-63);
//   B   one thread per pixel: the pixel's fragments in list order, found
//       through a per-pixel bit mask over the round's segments.
// A pixel covers ~4 of the ~25 pixels of a segment's box at 1080p, so the
// pair phases keep the lanes busy where a pixel-per-thread walk of the list
// would idle most of them.  Each slice of a pixel keeps the closed form of
// its front-to-back blend in registers: fragments arrive back to front
// (descending key) and acc = f + (1 - f.a) * acc, which equals the
// reference's per-slice linked list reduced front to back
// (reduceHairSlices.wgsl.ts:9-73) -- no fragment pool in memory.
//
// The reference's fragment-pool capacity per bin (SLICE_DATA_PER_PROCESSOR_
// COUNT, processHairSegment.wgsl.ts:33-40, hairFinePass.wgsl.ts:258-264) is
// kept exactly: while an upper bound (edge-test passes) shows that a bin
// cannot fill its pool inside a round, nothing is counted; otherwise the
// round is restricted to that bin, fragments are counted per segment, and the
// segment that fills the pool keeps its first slots in pixel order, after
// which the bin stops.
// ---------------------------------------------------------------------------
constexpr uint32_t NSHADE = 4;              // shading entries staged per segment
constexpr uint32_t MAX_RUNS = 66;           // runs of one round: at most one per depth bin (+1)
constexpr uint32_t EMPTY_BOX = 0x0000ffffu; // x0 = y0 = 255 > x1 = y1 = 0
constexpr uint32_t RUN_ENDS = 1u << 31;
constexpr uint32_t FINE_SPLIT_MIN = 256;  // records: tiles below this are never split

template <int TS> struct FineDims;
template <> struct FineDims<8> { static constexpr uint32_t STAGE = 64, PAIRS = 768; };
template <> struct FineDims<16> { static constexpr uint32_t STAGE = 128, PAIRS = 2048; };  // 96: 2-3 % slower, 160: 4 % slower
template <> struct FineDims<32> { static constexpr uint32_t STAGE = 256, PAIRS = 4096; };

// Shared inputs of the fine pass.
struct FineArgs {
  uint32_t S, P, B, L, SP, CAP, alphaQuadratic;
  float alphaMul;
  const float4* __restrict__ pos;
  const float4* __restrict__ tan;
  const float4* __restrict__ shading;
  const float* __restrict__ depth;
  const uint4* __restrict__ tiles;
  const uint32_t* __restrict__ segBuf;
  DeviceCounters* counters;
  const float4* __restrict__ proj;  // the tiles pass's projected segments (SEG_PROJ_VEC4 each), or NULL
};

template <int TS>
struct FineSmem {
  static constexpr uint32_t NT = TS * TS, STAGE = FineDims<TS>::STAGE, PAIRS = FineDims<TS>::PAIRS;
  static_assert(PAIRS >= NT, "a segment box covers up to TS*TS pairs");
  static_assert(2 * 6 * STAGE * sizeof(float) <= PAIRS * sizeof(uint2), "stagePoint's scratch fits in frag");
  float4 shade[STAGE][NSHADE];   // the shading entries each staged segment can sample
  uint2 frag[PAIRS];             // A1: pixel | segment << 16 of a passing pair; A2: its colour as 4 x f16
  uint32_t pairInfo[PAIRS];      // per box pair with a fragment (pixMask): fragment index | slice << 16
  // staged segments, one array per quantity (consecutive segments in consecutive banks)
  float ox[4][STAGE], oy[4][STAGE];  // first vertex of the four edge tests: v01, v11, v10, v00
  float ex[4][STAGE], ey[4][STAGE];  // second - first vertex of each edge test
  float dp[4][STAGE];                // depthsProj
  float qsx[STAGE], qsy[STAGE], qax[STAGE], qay[STAGE], qd2[STAGE], qlse[STAGE], qws[STAGE], qwe[STAGE],
      qd22[STAGE];                   // QuadConst
  uint32_t strand[STAGE], segIdx[STAGE], listIdx[STAGE];
  uint32_t box[STAGE];               // tile-local pixel box x0 | y0 << 8 | x1 << 16 | y1 << 24
  uint32_t shadeBase[STAGE];         // first staged shading index | count << 16 | depth bin << 24
  uint32_t pairBase[STAGE + 1];      // exclusive prefix of the box areas
  uint32_t rowBase[STAGE + 1];       // exclusive prefix of the box heights (A1's items)
  uint32_t cntEdge[STAGE], cntFrag[STAGE];
  uint32_t pixMask[STAGE / 32][NT];  // bit k of pixel p: staged segment k left a fragment at p
  // the tile
  uint4 head[64];                    // HairTileResult per depth bin
  float td0[64], td1[64];            // its depth range (_getTileDepth), for the slices of its fragments
  uint32_t binOff[65];               // tile mode: first entry of each bin in the tile's sequence
  float zbuf[NT];
  uint32_t doneMask[NT / 32];
  // the round
  uint32_t runBin[MAX_RUNS], runK0[MAX_RUNS], runK1[MAX_RUNS], runOff[MAX_RUNS];
  uint32_t red[32];
  // the work item's instance (written by one thread per item): read where used, so that none of
  // it stays in registers across the tile's rounds
  FineArgs args;
  uint32_t nRuns, nStaged, nSeg, passCount, queueIdx, bad, tileMode, total, walkNext;
  uint32_t mode, cutSeg, cutSlots, roundFrags, e0, eLast, arrive;
};

// Block-wide sum (all threads call; every thread gets the total).
template <int NW>
__device__ __forceinline__ uint32_t blockSum(uint32_t v, uint32_t* red, uint32_t lane, uint32_t warp) {
  const uint32_t w = __reduce_add_sync(0xffffffffu, v);
  if (lane == 0) red[warp] = w;
  __syncthreads();
  uint32_t t = 0;
#pragma unroll
  for (int i = 0; i < NW; i++) t += red[i];
  __syncthreads();
  return t;
}

// Block-wide exclusive prefix in thread order (all threads call).
template <int NW>
__device__ __forceinline__ uint32_t blockExclusive(uint32_t v, uint32_t* red, uint32_t lane, uint32_t warp) {
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) red[warp] = x;
  __syncthreads();
  uint32_t pre = 0;
  for (uint32_t i = 0; i < warp; i++) pre += red[i];
  __syncthreads();
  return pre + x - v;
}

// The shading entries staged segment (st, sg) can sample (tFull is
// monotonic in the segment coordinate, so they are [i0(t = 0), i1(t = 1)],
// at most NSHADE of them): loads them into sh.shade[k], returns
// first | count << 16.
template <int TS>
__device__ __forceinline__ uint32_t stageShade(FineSmem<TS>& sh, uint32_t k, uint32_t st, uint32_t sg,
                                               const float4* __restrict__ shading, uint32_t P, uint32_t SP) {
  uint32_t a0, a1, b0, b1;
  remapToIndices(SP, fadd((float)sg, 0.0f) / (float)(P - 1u), a0, a1);
  remapToIndices(SP, fadd((float)sg, 1.0f) / (float)(P - 1u), b0, b1);
  const uint32_t ne = min(b1 - a0 + 1u, NSHADE);
  const size_t sb = (size_t)st * SP;
  for (uint32_t j = 0; j < ne; j++) sh.shade[k][j] = __ldg(HFB_G(&shading[sb + a0 + j]));
  return a0 | (ne << 16);
}

// Staged segment k from its projection s: edge-test constants, depths, the
// pixel-independent part of interpolateHairQuad, and the tile-local box of
// the pixels that can pass the edge tests ([floor(min), ceil(max)] of the
// vertices).  shade: first | count << 16 of its staged shading entries
// (stageShade).  Returns the box area.
template <int TS>
__device__ __forceinline__ uint32_t stageFromProjection(FineSmem<TS>& sh, uint32_t k, uint32_t bin, const ProjSeg& s,
                                                        uint32_t shade, uint32_t x0, uint32_t y0) {
  uint32_t box = EMPTY_BOX, area = 0, shadeBase = bin << 24;
  float mnx = floorf(fminf(fminf(s.v00.x, s.v01.x), fminf(s.v10.x, s.v11.x))) - (float)x0;
  float mny = floorf(fminf(fminf(s.v00.y, s.v01.y), fminf(s.v10.y, s.v11.y))) - (float)y0;
  float mxx = ceilf(fmaxf(fmaxf(s.v00.x, s.v01.x), fmaxf(s.v10.x, s.v11.x))) - (float)x0;
  float mxy = ceilf(fmaxf(fmaxf(s.v00.y, s.v01.y), fmaxf(s.v10.y, s.v11.y))) - (float)y0;
  if (mnx <= mxx && mny <= mxy && mxx >= 0.0f && mxy >= 0.0f && mnx <= (float)(TS - 1) && mny <= (float)(TS - 1)) {
    const uint32_t bx0 = (uint32_t)fmaxf(mnx, 0.0f), by0 = (uint32_t)fmaxf(mny, 0.0f);
    const uint32_t bx1 = (uint32_t)fminf(mxx, (float)(TS - 1)), by1 = (uint32_t)fminf(mxy, (float)(TS - 1));
    box = bx0 | (by0 << 8) | (bx1 << 16) | (by1 << 24);
    area = (bx1 - bx0 + 1u) * (by1 - by0 + 1u);
    // edge tests in the order insideQuad evaluates them
    const f2 o[4] = {s.v01, s.v11, s.v10, s.v00};
    const f2 e[4] = {s.v00, s.v01, s.v11, s.v10};
#pragma unroll
    for (int i = 0; i < 4; i++) {
      sh.ox[i][k] = o[i].x;
      sh.oy[i][k] = o[i].y;
      sh.ex[i][k] = fsub(e[i].x, o[i].x);
      sh.ey[i][k] = fsub(e[i].y, o[i].y);
    }
    sh.dp[0][k] = s.depthsProj.x;
    sh.dp[1][k] = s.depthsProj.y;
    sh.dp[2][k] = s.depthsProj.z;
    sh.dp[3][k] = s.depthsProj.w;
    const QuadConst q = quadConst(s);
    sh.qsx[k] = q.sm.x; sh.qsy[k] = q.sm.y; sh.qax[k] = q.ab.x; sh.qay[k] = q.ab.y;
    sh.qd2[k] = q.d2; sh.qlse[k] = q.lse; sh.qws[k] = q.wS; sh.qwe[k] = q.wE; sh.qd22[k] = q.d22;
    shadeBase |= shade;
  }
  sh.box[k] = box;
  sh.shadeBase[k] = shadeBase;
  sh.cntEdge[k] = 0;
  sh.cntFrag[k] = 0;
  return area;
}

// Projects staged segment k (both points, projectSegment) and stages it.
template <int TS>
__device__ __forceinline__ uint32_t stageSegment(FineSmem<TS>& sh, uint32_t k, uint32_t bin, const HfbUniforms& U,
                                                 const float4* __restrict__ pos, const float4* __restrict__ tan,
                                                 const float4* __restrict__ shading, uint32_t S, uint32_t P,
                                                 uint32_t SP, f2 size, uint32_t x0, uint32_t y0) {
  const uint32_t st = sh.strand[k], sg = sh.segIdx[k];
  if (st < S && sg + 1u < P) {  // otherwise not a segment of this hair: covers no pixel
    const ProjSeg s = projectSegment(U, pos, tan, P, st, sg, size);
    return stageFromProjection<TS>(sh, k, bin, s, stageShade<TS>(sh, k, st, sg, shading, P, SP), x0, y0);
  }
  sh.box[k] = EMPTY_BOX;
  sh.shadeBase[k] = bin << 24;
  sh.cntEdge[k] = 0;
  sh.cntFrag[k] = 0;
  return 0u;
}

// Stages segment k from its projection in the tiles pass's cache.
template <int TS>
__device__ __forceinline__ uint32_t stageCached(FineSmem<TS>& sh, uint32_t k, uint32_t bin,
                                                const float4* __restrict__ proj, const float4* __restrict__ shading,
                                                uint32_t S, uint32_t P, uint32_t SP, uint32_t x0, uint32_t y0) {
  const uint32_t st = sh.strand[k], sg = sh.segIdx[k];
  if (st < S && sg + 1u < P) {
    const float4* q = proj + ((size_t)st * (P - 1u) + sg) * SEG_PROJ_VEC4;
    const float4 a = __ldg(HFB_G(&q[0])), b = __ldg(HFB_G(&q[1])), d = __ldg(HFB_G(&q[2]));
    ProjSeg s;
    s.v00 = mk2(a.x, a.y);
    s.v01 = mk2(a.z, a.w);
    s.v10 = mk2(b.x, b.y);
    s.v11 = mk2(b.z, b.w);
    s.depthsProj = mk4(d.x, d.y, d.z, d.w);
    return stageFromProjection<TS>(sh, k, bin, s, stageShade<TS>(sh, k, st, sg, shading, P, SP), x0, y0);
  }
  sh.box[k] = EMPTY_BOX;
  sh.shadeBase[k] = bin << 24;
  sh.cntEdge[k] = 0;
  sh.cntFrag[k] = 0;
  return 0u;
}

// With two threads per staged segment: thread `end` of segment k projects
// point sg + end of it (projectHairPoint) into the round's point scratch
// (the fragment list's storage, free until the edge tests); the end-point
// thread also stages the segment's shading entries.
template <int TS>
__device__ __forceinline__ void stagePoint(FineSmem<TS>& sh, uint32_t k, uint32_t end, const HfbUniforms& U,
                                           const float4* __restrict__ pos, const float4* __restrict__ tan,
                                           const float4* __restrict__ shading, uint32_t S, uint32_t P, uint32_t SP,
                                           f2 size) {
  constexpr uint32_t STAGE = FineSmem<TS>::STAGE;
  float* pt = reinterpret_cast<float*>(sh.frag) + end * 6u * STAGE;  // [6][STAGE] per end
  const uint32_t st = sh.strand[k], sg = sh.segIdx[k];
  if (!(st < S && sg + 1u < P)) return;
  const size_t i = (size_t)st * P + sg + end;
  f2 o0, o1;
  float z0, z1;
  projectHairPoint(U.modelMatrix.m, U.vpMatrix.m, mk3(U.cameraPosition.x, U.cameraPosition.y, U.cameraPosition.z),
                   ld4(__ldg(HFB_G(&pos[i]))), ld4(__ldg(HFB_G(&tan[i]))), size, U.fiberRadius, o0, o1, z0, z1);
  pt[0u * STAGE + k] = o0.x;
  pt[1u * STAGE + k] = o0.y;
  pt[2u * STAGE + k] = o1.x;
  pt[3u * STAGE + k] = o1.y;
  pt[4u * STAGE + k] = z0;
  pt[5u * STAGE + k] = z1;
  if (end) sh.shadeBase[k] = stageShade<TS>(sh, k, st, sg, shading, P, SP);
}

// Stages segment k from the two points stagePoint left.
template <int TS>
__device__ __forceinline__ uint32_t stageFromPoints(FineSmem<TS>& sh, uint32_t k, uint32_t bin, uint32_t S,
                                                    uint32_t P, uint32_t x0, uint32_t y0) {
  constexpr uint32_t STAGE = FineSmem<TS>::STAGE;
  const uint32_t st = sh.strand[k], sg = sh.segIdx[k];
  if (!(st < S && sg + 1u < P)) {
    sh.box[k] = EMPTY_BOX;
    sh.shadeBase[k] = bin << 24;
    sh.cntEdge[k] = 0;
    sh.cntFrag[k] = 0;
    return 0u;
  }
  const float* p0 = reinterpret_cast<const float*>(sh.frag);
  const float* p1 = p0 + 6u * STAGE;
  ProjSeg s;
  s.v00 = mk2(p0[0u * STAGE + k], p0[1u * STAGE + k]);
  s.v01 = mk2(p0[2u * STAGE + k], p0[3u * STAGE + k]);
  s.v10 = mk2(p1[0u * STAGE + k], p1[1u * STAGE + k]);
  s.v11 = mk2(p1[2u * STAGE + k], p1[3u * STAGE + k]);
  s.depthsProj = mk4(p0[4u * STAGE + k], p0[5u * STAGE + k], p1[4u * STAGE + k], p1[5u * STAGE + k]);
  return stageFromProjection<TS>(sh, k, bin, s, sh.shadeBase[k], x0, y0);
}

// Fragment colour of staged segment k at segment coordinates w and depth hd
// (processHairSegment.wgsl.ts:43-53 with getAlphaCoverage :60-69 and
// _sampleShading, hairShadingBuffer.ts:28-38), as 4 x f16, and its slice.
template <int TS>
__device__ __forceinline__ uint2 fragmentColour(const FineSmem<TS>& sh, uint32_t k, f2 w, float hd, uint32_t P,
                                                uint32_t SP, uint32_t L, float td0, float td1,
                                                uint32_t alphaQuadratic, float alphaMul,
                                                const float4* __restrict__ shading, uint32_t& slice) {
  float alpha = fsub(1.0f, fabsf(fsub(fmul(w.x, 2.0f), 1.0f)));
  if (alphaQuadratic) alpha = sqrtf(alpha);
  alpha = sat(fmul(alpha, alphaMul));
  const float tFull = fadd((float)sh.segIdx[k], w.y) / (float)(P - 1u);
  uint32_t i0, i1;
  const float fr = remapToIndices(SP, tFull, i0, i1);
  const uint32_t sbase = sh.shadeBase[k];
  const uint32_t e0 = sbase & 0xffffu, ne = (sbase >> 16) & 0xffu;
  float4 c0, c1;
  if (i0 - e0 < ne && i1 - e0 < ne) {
    c0 = sh.shade[k][i0 - e0];
    c1 = sh.shade[k][i1 - e0];
  } else {
    const size_t sb = (size_t)sh.strand[k] * SP;
    c0 = __ldg(HFB_G(&shading[sb + i0]));
    c1 = __ldg(HFB_G(&shading[sb + i1]));
  }
  f4 c = mix4(ld4(c0), ld4(c1), fr);
  c.w = fmul(c.w, alpha);
  slice = getDepthBin(L, td0, td1, hd);  // getSliceIdx
  const uint32_t hx = __half_as_ushort(__float2half_rn(c.x)), hy = __half_as_ushort(__float2half_rn(c.y));
  const uint32_t hz = __half_as_ushort(__float2half_rn(c.z)), hw = __half_as_ushort(__float2half_rn(c.w));
  return make_uint2(hx | (hy << 16), hz | (hw << 16));
}

__device__ __forceinline__ float halfLo(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v & 0xffffu))); }
__device__ __forceinline__ float halfHi(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v >> 16))); }

// acc[slice] = f + (1 - f.a) * acc[slice]
template <int MAXL>
__device__ __forceinline__ void blendFragment(f4 (&acc)[MAXL], uint32_t sl, uint2 h) {
  const f4 q = mk4(halfLo(h.x), halfHi(h.x), halfLo(h.y), halfHi(h.y));
  const float kk = fsub(1.0f, q.w);
#pragma unroll
  for (int si = 0; si < MAXL; si++) {
    if ((uint32_t)si == sl) {
      acc[si].x = fadd(q.x, fmul(kk, acc[si].x));
      acc[si].y = fadd(q.y, fmul(kk, acc[si].y));
      acc[si].z = fadd(q.z, fmul(kk, acc[si].z));
      acc[si].w = fadd(q.w, fmul(kk, acc[si].w));
    }
  }
}

// Tile mode: the runs of the next round, from bin `bin`, entry `off` of its
// list, up to `cap` segments.  Bins without depth (td1 == 0) are skipped as
// the reference skips them; a depth bin with an empty list is a run of zero
// segments (its reduce still runs).  Called by one thread.
template <int TS>
__device__ __forceinline__ uint32_t buildRuns(FineSmem<TS>& sh, uint32_t B, uint32_t bin, uint32_t off,
                                              uint32_t cap, uint32_t& used) {
  uint32_t n = 0;
  used = 0;
  while (bin < B && n < MAX_RUNS) {
    if (sh.head[bin].y == 0u) { bin++; off = 0; continue; }
    const uint32_t rem = sh.binOff[bin + 1] - sh.binOff[bin] - off;
    if (rem > 0u && used == cap) break;
    const uint32_t take = min(rem, cap - used);
    const bool ends = take == rem;
    sh.runBin[n] = bin | (ends ? RUN_ENDS : 0u);
    sh.runK0[n] = used;
    sh.runK1[n] = used + take;
    sh.runOff[n] = off;
    n++;
    used += take;
    if (!ends) break;
    bin++;
    off = 0;
  }
  return n;
}


// Rasterizes depth bins [b0, b1) of tile tileIdx in order, every pixel
// starting from an empty colour (processTile per bin + reduceHairSlices,
// hairFinePass.wgsl.ts:205-288), and leaves each pixel's colour in fin.
// With `independent`, the bins are a later part of a split tile: every pixel
// in view takes part, and the call gives up (returns false) as soon as a bin
// could fill its fragment pool, whose cut would depend on which pixels the
// earlier bins finished.
template <int TS, int MAXL>
__device__ __forceinline__ bool fineTile(FineSmem<TS>& sh, const HfbUniforms& U, const FineArgs& a,
                                         uint32_t tileIdx, uint32_t b0, uint32_t b1, bool independent, f4& fin) {
  using SM = FineSmem<TS>;
  constexpr uint32_t NT = SM::NT, STAGE = SM::STAGE, PAIRS = SM::PAIRS, NW = NT / 32u;
  constexpr uint32_t MODE_FAST = 0, MODE_TIGHTEN = 1, MODE_ABORT = 2;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t lx = tid % TS, ly = tid / TS;
  const f2 size = mk2(U.viewport.x, U.viewport.y);
  const uint32_t W = f2u(size.x), H = f2u(size.y);
  const uint32_t tilesX = divCeil(W, TS);
  const uint32_t maxDrawn = U.maxDrawnHairSegments;
  const uint32_t maxProcessed = a.S * a.P;  // MAX_PROCESSED_SEGMENTS, hairFinePass.wgsl.ts:212
  const uint32_t dispMode = U.displayMode & 0xffu;
  const uint32_t dbgMax = dispMode == 4u ? ((U.displayMode >> 8) & 0xffffu) : 0u;  // getDbgSlicesModeMaxSlices
  const bool isDbg = dbgMax != 0u;
  const uint32_t tx = tileIdx % tilesX, ty = tileIdx / tilesX;
  const TileB tbp = tileBoundsPx(W, H, TS, tx, ty);
  const uint32_t px = tbp.x0 + lx, py = tbp.y0 + ly;
  // Pixels of a partial edge tile outside the viewport take no part.
  const bool inView = px < W && py < H;
  sh.zbuf[tid] = inView ? loadTex2DClamp(a.depth, W, H, f2i((float)px), f2i(fsub(size.y, (float)py))) : 0.0f;
  bool done = !inView;
  {
    const uint32_t dm = __ballot_sync(0xffffffffu, done);
    if (lane == 0) sh.doneMask[warp] = dm;
  }
  fin = mk4(0.f, 0.f, 0.f, 0.f);  // rasterizerResult was cleared before the pass
  if (tid < a.B) {
    const uint4 h = (*HFB_G(&a.tiles[ty * tilesX * a.B + tx * a.B + tid]));
    sh.head[tid] = h;
    sh.td0[tid] = (float)(0xffffffffu - h.x) / F_MAX_U32;  // _getTileDepth
    sh.td1[tid] = (float)h.y / F_MAX_U32;
  }
  __syncthreads();

  // ---- tile mode: every depth bin's list carries a length hint (padding0,
  // written by the tiles pass) and the lists are the contiguous runs the
  // tiles pass writes; otherwise each list is walked ----
  if (warp == 0) {
    uint32_t ok = 1, sum = 0;
    for (uint32_t c0 = 0; c0 < a.B; c0 += 32) {
      const uint32_t bb = c0 + lane;
      uint32_t nb = 0;
      if (bb >= b0 && bb < b1) {
        const uint4 h = sh.head[bb];
        if (h.y != 0u && h.z != 0u) {
          if (h.w != 0u && h.w <= h.z && h.z <= maxDrawn && h.w <= maxProcessed) nb = h.w; else ok = 0;
        }
      }
      uint32_t incl = nb;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
      }
      if (bb < a.B) sh.binOff[bb] = sum + incl - nb;
      sum += __shfl_sync(0xffffffffu, incl, 31);
    }
    ok = __all_sync(0xffffffffu, ok);
    if (lane == 0) {
      sh.binOff[a.B] = sum;
      sh.total = sum;
      sh.tileMode = ok;
      sh.bad = 0;
    }
  }
  __syncthreads();
  bool tileMode = sh.tileMode != 0u;
  if (tileMode) {  // check every link of the contiguous layout
    const uint32_t total = sh.total;
    for (uint32_t k = tid; k < total; k += NT) {
      uint32_t lo = 0, hi = a.B;  // bin of k: binOff[lo] <= k < binOff[lo + 1]
      while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (sh.binOff[mid] <= k) lo = mid; else hi = mid;
      }
      const uint4 h = sh.head[lo];
      const uint32_t j = k - sh.binOff[lo];
      const uint32_t idx = h.z - 1u - j;
      if (!HFB_EXPECT(idx < maxDrawn)) { sh.bad = 1; continue; }
      const uint32_t nxt = __ldg(HFB_G(&a.segBuf[2u + 2u * idx]));
      if (nxt != ((j + 1u == h.w) ? INVALID_PTR : idx - 1u)) sh.bad = 1;
    }
    __syncthreads();
    tileMode = sh.bad == 0u;
  }

  // per-pixel state of the current bin
  f4 acc[MAXL];
#pragma unroll
  for (int si = 0; si < MAXL; si++) acc[si] = mk4(0.f, 0.f, 0.f, 0.f);
  uint32_t nFrag = 0, pending = 0;
  // uniform state: cursor and the pool accounting of the bin at the cursor
  uint32_t bin = b0, off = 0;                    // tile mode: bin, entry of its list
  uint32_t walkPtr = INVALID_PTR, processed = 0;  // walk mode: list pointer, entries processed
  uint32_t running = 0, runningUB = 0;            // slots taken (exact / upper bound)

  while (true) {
    // ---------------- stage the round ----------------
    if (tileMode) {
      if (tid == 0) {
        uint32_t used;
        sh.nRuns = buildRuns<TS>(sh, b1, bin, off, STAGE, used);
        sh.nStaged = used;
      }
      __syncthreads();
      const uint32_t nStaged = sh.nStaged, nRuns = sh.nRuns;
      for (uint32_t k = tid; k < nStaged; k += NT) {
        uint32_t r = 0;
        while (r + 1u < nRuns && sh.runK0[r + 1u] <= k) r++;
        const uint32_t b = sh.runBin[r] & 0xffu;
        const uint32_t idx = sh.head[b].z - 1u - (sh.runOff[r] + k - sh.runK0[r]);
        const uint32_t enc = HFB_EXPECT(idx < maxDrawn) ? __ldg(HFB_G(&a.segBuf[1u + 2u * idx])) : 0xffffffffu;
        sh.strand[k] = enc & 0x00ffffffu;
        sh.segIdx[k] = enc >> 24;
        sh.listIdx[k] = idx;
      }
    } else {
      while (bin < b1 && sh.head[bin].y == 0u) bin++;  // bins without depth are skipped
      if (bin >= b1) break;
      if (processed == 0u) {
        const uint32_t hz = sh.head[bin].z;
        walkPtr = hz == 0u ? INVALID_PTR : hz - 1u;
      }
      if (warp == 0) {  // speculative contiguous runs, else pointer chasing
        uint32_t p = walkPtr, m = 0;
        while (m < STAGE && p != INVALID_PTR && p < maxDrawn && processed + m < maxProcessed) {
          const uint32_t want = min(min(32u, STAGE - m), maxProcessed - processed - m);
          const uint32_t cand = p - lane;
          const bool inRange = lane < want && lane <= p;
          uint2 e = make_uint2(0u, INVALID_PTR);
          if (inRange) {
            e.x = __ldg(HFB_G(&a.segBuf[1u + 2u * cand]));
            e.y = __ldg(HFB_G(&a.segBuf[2u + 2u * cand]));
          }
          const bool chain = inRange && e.y == cand - 1u;
          const uint32_t brk = __ballot_sync(0xffffffffu, !chain);
          const uint32_t first = brk ? (uint32_t)(__ffs(brk) - 1) : 32u;
          bool firstIn = false;
          uint32_t firstNext = 0u;
          if (first < 32u) {
            firstIn = __shfl_sync(0xffffffffu, inRange, first);
            firstNext = __shfl_sync(0xffffffffu, e.y, first);
          }
          const uint32_t cnt = firstIn ? first + 1u : first;
          if (lane < cnt) {
            sh.strand[m + lane] = e.x & 0x00ffffffu;
            sh.segIdx[m + lane] = e.x >> 24;
            sh.listIdx[m + lane] = cand;
          }
          m += cnt;
          p = firstIn ? firstNext : p - cnt;
        }
        if (lane == 0) {
          const bool ends = !(p != INVALID_PTR && p < maxDrawn && processed + m < maxProcessed);
          sh.nStaged = m;
          sh.walkNext = p;
          sh.nRuns = 1;
          sh.runBin[0] = bin | (ends ? RUN_ENDS : 0u);
          sh.runK0[0] = 0;
          sh.runK1[0] = m;
          sh.runOff[0] = processed;
        }
      }
    }
    // In tile mode the runs were published at the barrier above and each thread
    // projects the segments it staged itself (the cached and the one-thread-per-
    // segment projections): no barrier is needed before the projection.
    if (!(tileMode && (a.proj != nullptr || 2u * STAGE > NT))) __syncthreads();
    uint32_t nRuns = sh.nRuns;
    if (nRuns == 0u) break;  // tile mode: no depth bin left
    const bool fresh = sh.runOff[0] == 0u;  // run 0 starts its bin
    if (fresh) { running = 0; runningUB = 0; }

    // ---------------- project ----------------
    {
      const uint32_t nStaged = sh.nStaged;
#pragma unroll
      for (uint32_t w = 0; w < STAGE / 32; w++) sh.pixMask[w][tid] = 0u;
      if (a.proj) {
        // the tiles pass projected every segment of the frame already
        for (uint32_t k = tid; k < nStaged; k += NT) {
          uint32_t r = 0;
          while (r + 1u < nRuns && sh.runK0[r + 1u] <= k) r++;
          sh.pairBase[k] = stageCached<TS>(sh, k, sh.runBin[r] & 0xffu, a.proj, a.shading, a.S, a.P, a.SP, tbp.x0,
                                           tbp.y0);
        }
      } else if constexpr (2u * STAGE <= NT) {
        // two threads per segment: one projects its first point, one its second
        if (tid < 2u * nStaged) {
          const uint32_t end = tid >= nStaged ? 1u : 0u;
          stagePoint<TS>(sh, tid - end * nStaged, end, U, a.pos, a.tan, a.shading, a.S, a.P, a.SP, size);
        }
        __syncthreads();
        for (uint32_t k = tid; k < nStaged; k += NT) {
          uint32_t r = 0;
          while (r + 1u < nRuns && sh.runK0[r + 1u] <= k) r++;
          sh.pairBase[k] = stageFromPoints<TS>(sh, k, sh.runBin[r] & 0xffu, a.S, a.P, tbp.x0, tbp.y0);
        }
      } else {
        for (uint32_t k = tid; k < nStaged; k += NT) {
          uint32_t r = 0;
          while (r + 1u < nRuns && sh.runK0[r + 1u] <= k) r++;
          sh.pairBase[k] = stageSegment<TS>(sh, k, sh.runBin[r] & 0xffu, U, a.pos, a.tan, a.shading, a.S, a.P,
                                            a.SP, size, tbp.x0, tbp.y0);
        }
      }
      __syncthreads();
      // exclusive prefix of the areas; the round keeps the longest prefix
      // of segments whose pairs fit
      if (warp == 0) {
        // the box areas (high half) and heights (low half) scanned together, all chunks of
        // 32 segments at once (independent shuffle chains); the halves cannot carry into each
        // other: at most STAGE * TS * TS and STAGE * TS, below 2^16 up to 16 px tiles
        using V = std::conditional_t<(TS <= 16), uint32_t, unsigned long long>;
        constexpr uint32_t SH = TS <= 16 ? 16u : 32u, NC = STAGE / 32u;
        constexpr V LOW = ((V)1 << SH) - 1u;
        V val[NC], incl[NC];
#pragma unroll
        for (uint32_t c = 0; c < NC; c++) {
          const uint32_t k = c * 32u + lane;
          const uint32_t a = k < nStaged ? sh.pairBase[k] : 0u;
          const uint32_t rows = a ? (sh.box[k] >> 24) - ((sh.box[k] >> 8) & 0xffu) + 1u : 0u;
          val[c] = ((V)a << SH) | rows;
          incl[c] = val[c];
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
          for (uint32_t c = 0; c < NC; c++) {
            const V y = __shfl_up_sync(0xffffffffu, incl[c], o);
            if (lane >= (uint32_t)o) incl[c] += y;
          }
        }
        V carryBoth = 0;
        uint32_t nSeg = nStaged;
#pragma unroll
        for (uint32_t c = 0; c < NC; c++) {
          const uint32_t k = c * 32u + lane;
          const V ex = carryBoth + incl[c] - val[c];
          if (k < nStaged) {
            sh.pairBase[k] = (uint32_t)(ex >> SH);
            sh.rowBase[k] = (uint32_t)(ex & LOW);
          }
          const uint32_t over =
              __ballot_sync(0xffffffffu, k < nStaged && (uint32_t)((carryBoth + incl[c]) >> SH) > PAIRS);
          if (over && nSeg == nStaged) nSeg = c * 32u + (uint32_t)(__ffs(over) - 1);
          carryBoth += __shfl_sync(0xffffffffu, incl[c], 31);
        }
        const uint32_t carry = (uint32_t)(carryBoth >> SH), carryRows = (uint32_t)(carryBoth & LOW);
        if (lane == 0) {
          sh.pairBase[nStaged] = carry;
          sh.rowBase[nStaged] = carryRows;
          sh.passCount = 0;
          if (nSeg < nStaged) {  // drop the segments from nSeg on
            if (tileMode) {
              uint32_t used;
              sh.nRuns = buildRuns<TS>(sh, b1, bin, off, nSeg, used);
            } else {
              sh.runK1[0] = nSeg;
              sh.runBin[0] &= ~RUN_ENDS;
            }
          }
          sh.nSeg = nSeg;
        }
      }
      __syncthreads();
    }
    uint32_t nSeg = sh.nSeg;
    nRuns = sh.nRuns;
    const uint32_t nPairs = sh.pairBase[nSeg];

    // ---------------- A1: edge tests, one thread per (segment, box row) ----------------
    // A thread tests every pixel of a box row (the row term of edgeFunction,
    // swRasterizeHair.wgsl.ts:128-130, formed once) into a bit mask, drops the
    // pixels that are done, and appends the rest with one shared atomic per warp.
    {
      const uint32_t nRows = sh.rowBase[nSeg];
      const uint32_t per = divCeil(nRows, NT);
      uint32_t it0 = tid * per;
      const uint32_t itEnd = min(it0 + per, nRows);
      uint32_t k = 0, ry = 0, myCnt = 0, bx0 = 0, bx1 = 0, by0 = 0, bh = 0;
      float eox[4], eey[4];
      auto loadSeg = [&](uint32_t kk) {
        const uint32_t bx = sh.box[kk];
        bx0 = bx & 0xffu;
        by0 = (bx >> 8) & 0xffu;
        bx1 = (bx >> 16) & 0xffu;
        bh = (bx >> 24) - by0 + 1u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
          eox[i] = sh.ox[i][kk]; eey[i] = sh.ey[i][kk];
        }
      };
      if (it0 < itEnd) {
        uint32_t lo = 0, hi = nSeg;  // last k with rowBase[k] <= it0
        while (hi - lo > 1u) {
          const uint32_t mid = (lo + hi) >> 1;
          if (sh.rowBase[mid] <= it0) lo = mid; else hi = mid;
        }
        k = lo;
        loadSeg(k);
        ry = it0 - sh.rowBase[k];
      }
      for (uint32_t it = 0; it < per; it++) {
        const bool valid = it0 < itEnd;
        uint32_t live = 0, rowPix = 0;
        if (valid) {
          const uint32_t qy = by0 + ry;
          const float py = (float)(tbp.y0 + qy);
          float rowT[4];
#pragma unroll
          for (int i = 0; i < 4; i++) rowT[i] = fmul(fsub(py, sh.oy[i][k]), sh.ex[i][k]);
          uint32_t bits = 0;
#pragma unroll
          for (uint32_t qx = 0; qx < (uint32_t)TS; qx++) {
            if (qx < bx0 || qx > bx1) continue;
            const float px = (float)(tbp.x0 + qx);
            bool pass = true;
#pragma unroll
            for (int i = 0; i < 4; i++) {  // edgeFunction >= 0
              const float C = fsub(fmul(fsub(px, eox[i]), eey[i]), rowT[i]);
              pass = pass && C >= 0.0f;
            }
            bits |= pass ? 1u << qx : 0u;
          }
          rowPix = qy * TS;
          const uint32_t rowDone = (sh.doneMask[rowPix >> 5] >> (rowPix & 31u)) &
                                   (TS == 32 ? 0xffffffffu : ((1u << (TS & 31)) - 1u));
          live = bits & ~rowDone;
        }
        // warp-aggregated append of the row's pixels
        const uint32_t n = (uint32_t)__popc(live);
        uint32_t incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t warpTotal = __shfl_sync(0xffffffffu, incl, 31);
        if (warpTotal) {
          uint32_t base = 0;
          if (lane == 31) base = atomicAdd(&sh.passCount, warpTotal);
          base = __shfl_sync(0xffffffffu, base, 31) + incl - n;
          while (live) {
            const uint32_t qx = (uint32_t)(__ffs(live) - 1);
            live &= live - 1u;
            if (HFB_EXPECT(base < PAIRS)) sh.frag[base].x = (rowPix + qx) | (k << 16);
            base++;
          }
        }
        myCnt += n;
        if (valid) {
          it0++;
          if (++ry == bh) {  // segment done
            if (myCnt) atomicAdd(&sh.cntEdge[k], myCnt);
            myCnt = 0;
            if (it0 < itEnd) {
              while (sh.rowBase[k + 1u] <= it0) k++;  // next segment with rows
              loadSeg(k);
              ry = 0;
            }
          }
        }
      }
      if (myCnt) atomicAdd(&sh.cntEdge[k], myCnt);
    }
    __syncthreads();

    // ---------------- can a bin fill its pool in this round? ----------------
    // The edge-test passes bound the fragments: when the passes of the whole
    // round, on top of what the cursor's bin may already hold, fit in a pool,
    // no bin can fill its pool and nothing needs counting (the common case:
    // every thread sees passCount after the barrier above).  Otherwise one
    // warp sums the passes run by run.  e0 / eLast carry the bounds of the
    // first and last run (the round's total where it is enough).
    uint32_t mode = MODE_FAST, e0 = sh.passCount, eLast = e0;
    if (runningUB + e0 > a.CAP) {
      if (warp == 0) {
        uint32_t wmode = MODE_FAST, keep = nRuns, we0 = 0, weLast = 0;
        for (uint32_t r = 0; r < nRuns; r++) {
          uint32_t e = 0;
          for (uint32_t k = sh.runK0[r] + lane; k < sh.runK1[r]; k += 32) e += sh.cntEdge[k];
          e = __reduce_add_sync(0xffffffffu, e);
          const uint32_t base = r == 0u ? runningUB : 0u;
          if (r == 0u) we0 = e;
          if (base + e > a.CAP) {
            if (r == 0u) { wmode = MODE_TIGHTEN; keep = 1; } else { keep = r; }
            break;
          }
          weLast = e;
        }
        if (independent && (wmode == MODE_TIGHTEN || keep < nRuns)) wmode = MODE_ABORT;
        if (lane == 0) {
          sh.mode = wmode;
          sh.e0 = we0;
          sh.eLast = weLast;
          if (keep < nRuns) {  // the round ends where that bin's run starts
            sh.nRuns = keep;
            sh.nSeg = sh.runK1[keep - 1u];
          }
          sh.roundFrags = 0;
        }
      }
      __syncthreads();
      mode = sh.mode;
      e0 = sh.e0;
      eLast = sh.eLast;
      if (mode == MODE_ABORT) return false;  // a pool could fill: this group cannot stand alone
      nRuns = sh.nRuns;
      nSeg = sh.nSeg;
    }
    bool exact = false;
    if (mode == MODE_TIGHTEN) {
      running += blockSum<NW>(pending, sh.red, lane, warp);
      pending = 0;
      runningUB = running;
      exact = runningUB + e0 > a.CAP;
    }

    // ---------------- A2: fragments, one thread per passing pair ----------------
    {
      // the arguments this phase reads, in registers for the phase only
      const uint32_t P = a.P, SP = a.SP, L = a.L, alphaQuadratic = a.alphaQuadratic;
      const float alphaMul = a.alphaMul;
      const float4* __restrict__ shading = a.shading;
      const uint32_t nPass = sh.passCount;
      for (uint32_t i = tid; i < nPass; i += NT) {
        const uint32_t e = sh.frag[i].x;
        const uint32_t pix = e & 0xffffu, k = e >> 16;
        if (k >= nSeg) continue;  // dropped from the round
        if (!HFB_EXPECT(i < PAIRS && k < STAGE && pix < NT)) continue;
        const uint32_t qx = pix % TS, qy = pix / TS;
        const f2 pf = mk2((float)(tbp.x0 + qx), (float)(tbp.y0 + qy));
        QuadConst qc;
        qc.sm = mk2(sh.qsx[k], sh.qsy[k]);
        qc.ab = mk2(sh.qax[k], sh.qay[k]);
        qc.d2 = sh.qd2[k]; qc.lse = sh.qlse[k]; qc.wS = sh.qws[k]; qc.wE = sh.qwe[k];
        qc.ab2 = mk2(sh.ex[3][k], sh.ey[3][k]);
        qc.d22 = sh.qd22[k];
        const f2 w = interpolateHairQuadPre(qc, mk2(sh.ox[3][k], sh.oy[3][k]), pf);
        const float hd = interpolateHairF32(w, mk4(sh.dp[0][k], sh.dp[1][k], sh.dp[2][k], sh.dp[3][k]));
        if (!(hd < sh.zbuf[pix])) continue;  // depth test with GL_LESS (skip when >=)
        const uint32_t kb = sh.shadeBase[k] >> 24;
        const float td0 = sh.td0[kb], td1 = sh.td1[kb];
        uint32_t slice;
        const uint2 col = fragmentColour<TS>(sh, k, w, hd, P, SP, L, td0, td1, alphaQuadratic, alphaMul, shading,
                                             slice);
        sh.frag[i] = col;
        const uint32_t bx = sh.box[k];
        sh.pairInfo[sh.pairBase[k] + (qy - ((bx >> 8) & 0xffu)) * (((bx >> 16) & 0xffu) - (bx & 0xffu) + 1u) +
                    (qx - (bx & 0xffu))] = i | (slice << 16);
        atomicOr(&sh.pixMask[k >> 5][pix], 1u << (k & 31u));
        if (exact) atomicAdd(&sh.cntFrag[k], 1u);
      }
    }
    __syncthreads();

    // ---------------- exact accounting: the segment that fills the pool ----------------
    if (exact) {
      if (warp == 0) {  // one run (this bin) in the round
        uint32_t carry = 0, cut = INVALID_PTR, cutSlots = 0;
        for (uint32_t k0 = 0; k0 < nSeg; k0 += 32) {
          const uint32_t k = k0 + lane;
          const uint32_t c = k < nSeg ? sh.cntFrag[k] : 0u;
          uint32_t incl = c;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
          }
          const uint32_t fb = __ballot_sync(0xffffffffu, k < nSeg && running + carry + incl >= a.CAP);
          if (fb) {
            const uint32_t j = (uint32_t)(__ffs(fb) - 1);
            cut = k0 + j;
            cutSlots = a.CAP - (running + carry + __shfl_sync(0xffffffffu, incl - c, j));
            break;
          }
          carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) {
          sh.cutSeg = cut;
          sh.cutSlots = cutSlots;
          sh.roundFrags = carry;
          if (cut != INVALID_PTR) {
            sh.nSeg = cut + 1u;
            sh.runK1[0] = cut + 1u;
            sh.runBin[0] |= RUN_ENDS;  // the reference breaks after the filling segment
            atomicAdd(HFB_G(&a.counters->finePoolFullBins), 1ull);
          }
        }
      }
      __syncthreads();
      const uint32_t cut = sh.cutSeg;
      if (cut != INVALID_PTR) {  // slots of the filling segment in pixel order
        const uint32_t b = sh.box[cut], bxa = b & 0xffu, bya = (b >> 8) & 0xffu;
        const uint32_t bw = ((b >> 16) & 0xffu) - bxa + 1u, area = sh.pairBase[cut + 1u] - sh.pairBase[cut];
        const uint32_t pix = tid < area ? (bya + tid / bw) * TS + bxa + tid % bw : 0u;
        const uint32_t bit = 1u << (cut & 31u);
        const bool has = tid < area && (sh.pixMask[cut >> 5][pix] & bit) != 0u;
        const uint32_t rank = blockExclusive<NW>(has ? 1u : 0u, sh.red, lane, warp);
        if (has && rank >= sh.cutSlots) sh.pixMask[cut >> 5][pix] &= ~bit;  // the pool is full
        __syncthreads();
      }
      nSeg = sh.nSeg;
    }

    // ---------------- B: every pixel blends its fragments in list order ----------------
    const uint32_t L = a.L;
    for (uint32_t r = 0; r < nRuns; r++) {
      const uint32_t rb = sh.runBin[r], k0 = sh.runK0[r], k1 = sh.runK1[r];
      if (!done && k0 < k1) {
        for (uint32_t w = k0 >> 5; w <= (k1 - 1u) >> 5; w++) {
          const uint32_t lo = max(k0, w * 32u) - w * 32u, hi = min(k1, w * 32u + 32u) - w * 32u;
          uint32_t bits = sh.pixMask[w][tid] & (hi == 32u ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
          while (bits) {
            const uint32_t j = w * 32u + (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1u;
            const uint32_t b = sh.box[j];
            const uint32_t bx0 = b & 0xffu, by0 = (b >> 8) & 0xffu;
            const uint32_t info =
                sh.pairInfo[sh.pairBase[j] + (ly - by0) * (((b >> 16) & 0xffu) - bx0 + 1u) + (lx - bx0)];
            if (HFB_EXPECT((info & 0xffffu) < PAIRS)) {
              blendFragment<MAXL>(acc, info >> 16, sh.frag[info & 0xffffu]);
              nFrag++;
              pending++;
            }
          }
        }
      }
      if (rb & RUN_ENDS) {
        // reduceHairSlices (runs for every bin with depth, as in the reference)
        if (!done) {
          if (isDbg) {
            const uint32_t cntAll = f2u(fmul(fin.x, (float)dbgMax)) + nFrag;
            fin = mk4(sat((float)cntAll / (float)dbgMax), 0.0f, 0.0f, 1.0f);
          } else {
#pragma unroll
            for (int si = 0; si < MAXL; si++) {
              if ((uint32_t)si < L && fin.w < 0.999f) {
                const float kk = fsub(1.0f, fin.w);
                fin.x = fadd(fin.x, fmul(acc[si].x, kk));
                fin.y = fadd(fin.y, fmul(acc[si].y, kk));
                fin.z = fadd(fin.z, fmul(acc[si].z, kk));
                fin.w = fadd(fin.w, fmul(acc[si].w, kk));
              }
            }
            done = fin.w >= 0.999f;  // isPixelDone with ALPHA_CUTOFF
          }
        }
#pragma unroll
        for (int si = 0; si < MAXL; si++) acc[si] = mk4(0.f, 0.f, 0.f, 0.f);
        nFrag = 0;
        pending = 0;
      }
    }

    // ---------------- carry the pool state and advance the cursor ----------------
    const uint32_t lastBin = sh.runBin[nRuns - 1u];
    const bool lastEnds = (lastBin & RUN_ENDS) != 0u;
    if (lastEnds) {
      running = 0;
      runningUB = 0;
    } else if (nRuns == 1u) {
      if (exact) {
        running += sh.roundFrags;
        runningUB = running;
        pending = 0;
      } else {
        runningUB += e0;
      }
    } else {
      running = 0;
      runningUB = eLast;
    }
    if (tileMode) {
      const uint32_t lb = lastBin & 0xffu;
      if (lastEnds) { bin = lb + 1u; off = 0; }
      else { off = sh.runOff[nRuns - 1u] + sh.runK1[nRuns - 1u] - sh.runK0[nRuns - 1u]; bin = lb; }
    } else {
      if (lastEnds) { bin++; processed = 0; }
      else {
        walkPtr = nSeg < sh.nStaged ? sh.listIdx[nSeg] : sh.walkNext;
        processed += nSeg;
      }
    }
    {
      const uint32_t dm = __ballot_sync(0xffffffffu, done);
      if (lane == 0) sh.doneMask[warp] = dm;
    }
    // checkAllPixelsInWkgrpDone, :305-327 (also the barrier before the
    // next round rewrites the staged state)
    if (__syncthreads_and(done)) break;
    if (bin >= b1) break;
  }
  return true;
}

// Builds the work list of the fine pass: one item per drawn tile, in the
// tile list's order (most records first), except that a tile with more
// records than a CTA's average share is split into groups of whole depth
// bins, so that no single CTA carries the frame's tail.  Group sizes come
// from the list-length hints; a tile without valid hints is not split.
// One CTA.
__device__ __forceinline__ void fineScheduleBody(const uint32_t* __restrict__ tileList,
                                                 const uint32_t* __restrict__ segCount,
                                                 const uint4* __restrict__ tiles, uint32_t T, uint32_t B,
                                                 uint32_t grid, uint32_t maxDrawn, uint32_t maxProcessed,
                                                 uint32_t allowSplit, const FineScratch& fs,
                                                 DeviceCounters* __restrict__ counters, uint32_t* warpSums,
                                                 uint32_t& total) {
  const uint32_t tid = threadIdx.x;
  const uint32_t drawn = min((*HFB_G(&tileList[0])), T);
  if (tid == 0) total = 0;
  __syncthreads();
  uint32_t mine = 0;
  for (uint32_t q = tid; q < drawn; q += blockDim.x) {
    const uint32_t t = (*HFB_G(&tileList[1u + q]));
    if (t < T) mine += (*HFB_G(&segCount[t]));
  }
  atomicAdd(&total, mine);
  __syncthreads();
  const uint32_t thr = max(FINE_SPLIT_MIN, total / max(grid, 1u));
  uint32_t carryItems = 0, carrySlots = 0;
  for (uint32_t q0 = 0; q0 < drawn; q0 += blockDim.x) {
    const uint32_t q = q0 + tid;
    uint32_t nG = 0, t = T;  // items of this tile-list entry: none past the list's end
    if (q < drawn) {
      nG = 1;
      t = (*HFB_G(&tileList[1u + q]));
      if (allowSplit && t < T && (*HFB_G(&segCount[t])) > thr) {  // count the groups of the split
        uint32_t g = 0, acc = 0;
        bool ok = true;
        for (uint32_t b = 0; b < B; b++) {
          const uint4 h = (*HFB_G(&tiles[(size_t)t * B + b]));
          uint32_t nb = 0;
          if (h.y != 0u && h.z != 0u) {
            if (h.w != 0u && h.w <= h.z && h.z <= maxDrawn && h.w <= maxProcessed) nb = h.w; else ok = false;
          }
          if (nb == 0u) continue;
          if (acc > 0u && acc + nb > thr) { g++; acc = 0; }
          acc += nb;
        }
        if (acc > 0u) g++;
        if (ok && g > 1u) nG = g;
      }
    }
    uint32_t chunkSlots;
    const uint32_t mySlots = nG > 1u ? nG : 0u;
    const uint32_t slotEnd = carrySlots + blockExclusiveScan(mySlots, warpSums, chunkSlots) + mySlots;
    const bool split = nG > 1u && slotEnd <= fs.maxGroups;
    if (nG > 1u && !split) nG = 1;
    uint32_t chunkItems;
    const uint32_t itemBase = carryItems + blockExclusiveScan(nG, warpSums, chunkItems);
    if (q < drawn) {
      if (split) {
        const uint32_t slot = slotEnd - nG;
        (*HFB_G(&fs.arrivals[slot])) = 0;
        atomicAdd(HFB_G(&counters->fineSplitTiles), 1ull);
        uint32_t g = 0, acc = 0, start = 0;
        for (uint32_t b = 0; b < B; b++) {
          const uint4 h = (*HFB_G(&tiles[(size_t)t * B + b]));
          const uint32_t nb = (h.y != 0u && h.z != 0u) ? h.w : 0u;
          if (nb == 0u) continue;
          if (acc > 0u && acc + nb > thr) {
            (*HFB_G(&fs.items[itemBase + g])) = make_uint4(q, start | (b << 8) | (g << 16) | (nG << 24), slot, 0u);
            g++;
            acc = 0;
            start = b;
          }
          acc += nb;
        }
        (*HFB_G(&fs.items[itemBase + g])) = make_uint4(q, start | (B << 8) | (g << 16) | (nG << 24), slot, 0u);
      } else {
        (*HFB_G(&fs.items[itemBase])) = make_uint4(q, 0u | (B << 8) | (1u << 24), 0u, 0u);
      }
    }
    carryItems += chunkItems;
    carrySlots += chunkSlots;
  }
  if (tid == 0) (*HFB_G(&fs.hdr[0])) = carryItems;
  __syncthreads();
}

__global__ void __launch_bounds__(1024)
fineScheduleKernel(const uint32_t* __restrict__ tileList, const uint32_t* __restrict__ segCount,
                   const uint4* __restrict__ tiles, uint32_t T, uint32_t B, uint32_t grid, uint32_t maxDrawn,
                   uint32_t maxProcessed, uint32_t allowSplit, FineScratch fs,
                   DeviceCounters* __restrict__ counters) {
  __shared__ uint32_t warpSums[32];
  __shared__ uint32_t total;
  fineScheduleBody(tileList, segCount, tiles, T, B, grid, maxDrawn, maxProcessed, allowSplit, fs, counters,
                   warpSums, total);
}

// One work item of the fine pass: a tile, or one group of depth bins of a
// split tile (then the last group to finish merges the tile).
template <int TS, int MAXL>
__device__ __forceinline__ void fineItem(FineSmem<TS>& sh, const HfbUniforms& U, const FineArgs& a,
                                         const uint32_t* __restrict__ tileList, float* __restrict__ result,
                                         const FineScratch fs, const uint4 item) {
  using SM = FineSmem<TS>;
  constexpr uint32_t NT = SM::NT;
  constexpr uint32_t UNSAFE = 1u << 31;
  const uint32_t tid = threadIdx.x;
  const uint32_t lx = tid % TS, ly = tid / TS;
  const uint32_t W = f2u(U.viewport.x), H = f2u(U.viewport.y);
  const uint32_t tilesX = divCeil(W, TS), tileCount = tilesX * divCeil(H, TS);
  float4* res = reinterpret_cast<float4*>(result + 4);
  {
    if (item.x >= tileCount) {  // not an entry of the tile list: count it and skip
      if (tid == 0) atomicAdd(HFB_G(&a.counters->badWorkItems), 1ull);
      return;
    }
    const uint32_t tileIdx = (*HFB_G(&tileList[1u + item.x]));
    uint32_t b0 = item.y & 0xffu, b1 = (item.y >> 8) & 0xffu;
    const uint32_t g = (item.y >> 16) & 0xffu, nG = item.y >> 24;
    if (tileIdx >= tileCount || b1 > a.B || b0 >= b1) return;
    bool split = nG > 1u, write = true;
    if (split && (g >= nG || item.z >= fs.maxGroups || nG > fs.maxGroups - item.z)) {
      // not an item the schedule writes: count it and leave the tile alone
      if (tid == 0) atomicAdd(HFB_G(&a.counters->badWorkItems), 1ull);
      return;
    }
    f4 fin;
    while (true) {
      const bool ok = fineTile<TS, MAXL>(sh, U, a, tileIdx, b0, b1, split && g > 0u, fin);
      if (!split) break;
      // a group of a split tile: publish its composite; the last to arrive merges
      (*HFB_G(&fs.groups[(size_t)(item.z + g) * NT + tid])) = make_float4(fin.x, fin.y, fin.z, fin.w);
      __threadfence();
      __syncthreads();
      if (tid == 0) {
        if (!ok) atomicOr(HFB_G(&fs.arrivals[item.z]), UNSAFE);
        const uint32_t old = atomicAdd(HFB_G(&fs.arrivals[item.z]), 1u);
        sh.arrive = (old & 0xffffu) + 1u == nG ? ((old & UNSAFE) ? 2u : 1u) : 0u;
        if (sh.arrive == 2u) atomicAdd(HFB_G(&a.counters->fineSplitRedone), 1ull);
      }
      __syncthreads();
      const uint32_t m = sh.arrive;
      if (m == 0u) { write = false; break; }
      if (m == 2u) {  // a later group could fill a pool: the whole tile in order
        b0 = 0;
        b1 = a.B;
        split = false;
        continue;
      }
      __threadfence();
      // front-to-back "over" of the groups' composites, each pixel stopping
      // where the reference stops (isPixelDone, alpha >= 0.999)
      const float4 f0 = __ldcg(HFB_G(&fs.groups[(size_t)item.z * NT + tid]));
      fin = mk4(f0.x, f0.y, f0.z, f0.w);
      for (uint32_t g2 = 1; g2 < nG; g2++) {
        const float4 c = __ldcg(HFB_G(&fs.groups[(size_t)(item.z + g2) * NT + tid]));
        if (fin.w < 0.999f) {
          const float k = fsub(1.0f, fin.w);
          fin.x = fadd(fin.x, fmul(c.x, k));
          fin.y = fadd(fin.y, fmul(c.y, k));
          fin.z = fadd(fin.z, fmul(c.z, k));
          fin.w = fadd(fin.w, fmul(c.w, k));
        }
      }
      break;
    }
    const uint32_t tx = tileIdx % tilesX, ty = tileIdx / tilesX;
    const TileB tbp = tileBoundsPx(W, H, TS, tx, ty);
    const uint32_t px = tbp.x0 + lx, py = tbp.y0 + ly;
    if (write && px < W && py < H) (*HFB_G(&res[(size_t)py * W + px])) = make_float4(fin.x, fin.y, fin.z, fin.w);
  }
}

template <int TS, int MAXL>
__global__ void __launch_bounds__(TS * TS, TS == 8 ? (MAXL <= 4 ? 8 : 6) : TS == 16 ? (MAXL <= 4 ? 3 : 2) : 1)
fineKernel(const HfbUniforms U, const FineArgs a, const uint32_t* __restrict__ tileList, float* __restrict__ result,
           FineScratch fs) {
  using SM = FineSmem<TS>;
  extern __shared__ __align__(16) unsigned char fineSmemRaw[];
  SM& sh = *reinterpret_cast<SM*>(fineSmemRaw);
  const uint32_t nItems = min((*HFB_G(&fs.hdr[0])), fs.maxItems);
  uint32_t* queue = reinterpret_cast<uint32_t*>(result);  // tileQueueAtomicIdx, getNextTileIdx :294-303
  // The device functions get the uniforms and the arguments from shared
  // memory, never an address of a kernel parameter (whose generic address
  // lies in the parameter space, which instructions for global memory
  // reject: error 717, invalid address space).
  __shared__ HfbUniforms Us;
  for (uint32_t w = threadIdx.x; w < sizeof(HfbUniforms) / 4u; w += blockDim.x)
    reinterpret_cast<uint32_t*>(&Us)[w] = reinterpret_cast<const uint32_t*>(&U)[w];
  if (threadIdx.x == 0) sh.args = a;
  while (true) {
    if (threadIdx.x == 0) sh.queueIdx = atomicAdd(HFB_G(queue), 1u);
    __syncthreads();
    const uint32_t it = sh.queueIdx;
    if (it >= nItems) break;
    fineItem<TS, MAXL>(sh, Us, sh.args, tileList, result, fs, (*HFB_G(&fs.items[it])));
    __syncthreads();  // the tile's shared state is rewritten for the next item
  }
}

// batched: one queue over the work items of every instance
template <int TS, int MAXL>
__global__ void __launch_bounds__(TS * TS, TS == 8 ? (MAXL <= 4 ? 8 : 6) : TS == 16 ? (MAXL <= 4 ? 3 : 2) : 1)
fineBatch(BatchView b, FineArgs base, HfbConfig cfgParam) {
  using SM = FineSmem<TS>;
  const HfbConfig cfg = cfgParam;
  extern __shared__ __align__(16) unsigned char fineSmemRaw[];
  SM& sh = *reinterpret_cast<SM*>(fineSmemRaw);
  const uint32_t n = b.hdr->n;
  const uint32_t total = b.itemPrefix[n];
  while (true) {
    if (threadIdx.x == 0) {
      const uint32_t gi = atomicAdd(&b.hdr->fineQueue, 1u);
      sh.queueIdx = gi;
      if (gi < total) {  // the item's instance, for every thread of the CTA
        const BatchInst& I = b.insts[batchFind(b.itemPrefix, n, gi)];
        FineArgs a = base;
        a.S = I.S;
        a.P = I.P;
        a.pos = I.posNew;
        a.tan = I.tan;
        a.shading = I.shading;
        a.depth = I.depth;
        a.tiles = I.tiles;
        a.segBuf = I.segBuf;
        a.proj = I.proj;
        sh.args = a;
      }
    }
    __syncthreads();
    const uint32_t gi = sh.queueIdx;
    if (gi >= total) break;
    const uint32_t i = batchFind(b.itemPrefix, n, gi);
    const BatchInst& I = b.insts[i];
    const FineScratch fs = fineScratchLayout(I.scratch, cfg, I.W, I.H);
    const uint32_t li = gi - b.itemPrefix[i];
    if (li < fs.maxItems) fineItem<TS, MAXL>(sh, I.U, sh.args, I.tileList, I.result, fs, (*HFB_G(&fs.items[li])));
    __syncthreads();
  }
}

template <int TS, int MAXL>
cudaError_t launchFineT(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                        const float* tan, const float* shading, const float* depth, HfbRasterBuffers& rb,
                        const float4* proj) {
  HFB_CHECK_BIND(c);
  const HfbConfig& cfg = c->cfg;
  constexpr size_t SMEM = sizeof(FineSmem<TS>);
  int& perSM = c->fineBlocksPerSM[TS == 8 ? 0 : TS == 16 ? 1 : 2][MAXL == 4 ? 0 : MAXL == 8 ? 1 : 2];
  if (perSM == 0) {
    cudaError_t e = cudaFuncSetAttribute(fineKernel<TS, MAXL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fineKernel<TS, MAXL>, TS * TS, SMEM);
    if (e != cudaSuccess) return e;
    if (perSM < 1) return cudaErrorInvalidConfiguration;
  }
  const uint32_t grid = cfg.processorCount ? cfg.processorCount : (uint32_t)(perSM * c->smCount);
  const uint32_t T = divCeil(rb.width, TS) * divCeil(rb.height, TS);
  const uint32_t dispMode = u.displayMode & 0xffu;
  const bool dbg = dispMode == 4u && ((u.displayMode >> 8) & 0xffffu) != 0u;
  FineScratch fs = fineScratchLayout(rb.scratch, cfg, rb.width, rb.height);
  fineScheduleKernel<<<1, 1024, 0, c->stream>>>(rb.tileList, rb.segmentCountPerTile, (const uint4*)rb.tiles, T,
                                                cfg.tileDepthBins, grid, rb.maxDrawnSegments,
                                                h.strandsCount * h.pointsPerStrand, dbg ? 0u : 1u, fs,
                                                (DeviceCounters*)c->dCounters);
  HFB_AFTER_LAUNCH(c, "fineScheduleKernel");
  FineArgs a;
  a.S = h.strandsCount;
  a.P = h.pointsPerStrand;
  a.B = cfg.tileDepthBins;
  a.L = cfg.slicesPerPixel;
  a.SP = cfg.shadingPoints;
  a.CAP = cfg.avgFragmentsPerSlice * cfg.slicesPerPixel * cfg.tileSize * cfg.tileSize;
  a.alphaQuadratic = cfg.alphaQuadratic;
  a.alphaMul = cfg.alphaMultiplier;
  a.pos = (const float4*)pos;
  a.tan = (const float4*)tan;
  a.shading = (const float4*)shading;
  a.depth = depth;
  a.tiles = (const uint4*)rb.tiles;
  a.segBuf = rb.tileSegments;
  a.counters = (DeviceCounters*)c->dCounters;
  a.proj = proj;
  fineKernel<TS, MAXL><<<grid, TS * TS, SMEM, c->stream>>>(u, a, rb.tileList, rb.rasterizerResult, fs);
  HFB_AFTER_LAUNCH(c, "fineKernel");
  c->launches += 2;
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Batched tiles pass, tile sort and fine pass: persistent over the virtual
// blocks of every instance (hfb_frame_batch).
// ---------------------------------------------------------------------------
#define BATCH_LOOP(KIND)                                              \
  const uint32_t n = b.hdr->n;                                        \
  const uint32_t* row = b.prefix + (KIND) * (BATCH_MAX + 1);          \
  const uint32_t totalVb = row[n];                                    \
  __shared__ uint32_t vbNext[2];                                      \
  uint32_t vbPar = 0;                                                 \
  for (uint32_t v = batchNext(b.hdr, (KIND), vbNext, vbPar); v < totalVb; \
       v = batchNext(b.hdr, (KIND), vbNext, vbPar)) {                 \
    const uint32_t i = batchFind(row, n, v);                          \
    const BatchInst& I = b.insts[i];                                  \
    if (!HFB_EXPECT(i < n && I.W && I.H && I.W <= 65536 && I.H <= 65536 && I.scratch && I.segBuf && \
                    I.T == divCeil(I.W, cfg.tileSize) * divCeil(I.H, cfg.tileSize))) continue; \
    const uint32_t local = v - row[i], nLocal = row[i + 1] - row[i];  \
    (void)nLocal; (void)local;                                        \
    const TilesScratch ts = tilesScratchLayout(I.scratch, cfg, I.W, I.H, I.maxDrawn); \
    (void)ts;

__global__ void __launch_bounds__(TR_SEGS, 7) tilesRasterBatch(BatchView b, HfbConfig cfgParam,
                                                             DeviceCounters* __restrict__ counters) {
  const HfbConfig cfg = cfgParam;
  __shared__ TrShared<TR_SLOTS_BATCH, TR_CHUNK_BATCH> sh;
  BATCH_LOOP(BK_RASTER)
    tilesRasterBody<TR_SLOTS_BATCH, TR_CHUNK_BATCH>(I.U, I.P, min(I.strandsToRender, I.S), cfg.tileSize, cfg.tileDepthBins,
                    cfg.invalidTilesPerSegmentThreshold, I.bsphere, I.posNew, I.tan, I.depth, I.tiles, I.segBuf,
                    I.segCount, ts.binCount, counters, sh, local, I.proj);
  }
}

__global__ void __launch_bounds__(512) binScanBatch(BatchView b, HfbConfig cfgParam) {
  const HfbConfig cfg = cfgParam;
  __shared__ uint32_t warpSums[32];
  BATCH_LOOP(BK_SCAN)
    binScanBlocksBody(ts.binCount, ts.binOffset, ts.blockSums, I.T * cfg.tileDepthBins, warpSums, local);
  }
}

__global__ void __launch_bounds__(1024) binScanSumsBatch(BatchView b, HfbConfig cfgParam) {
  const HfbConfig cfg = cfgParam;
  __shared__ uint32_t warpSums[32];
  BATCH_LOOP(BK_SCAN_SUMS)
    binScanSumsBody(ts.blockSums, divCeil(I.T * cfg.tileDepthBins, SCAN_PER_BLOCK), warpSums);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) binScatterBatch(BatchView b, HfbConfig cfgParam,
                                                        DeviceCounters* __restrict__ counters) {
  const HfbConfig cfg = cfgParam;
  BATCH_LOOP(BK_SCATTER)
    binScatterBody(I.segBuf, I.maxDrawn, ts.binOffset, ts.blockSums, ts.keys, counters, local, nLocal,
                   I.T * cfg.tileDepthBins);
  }
}

__global__ void __launch_bounds__(256) binFinalizeBatch(BatchView b, HfbConfig cfgParam) {
  const HfbConfig cfg = cfgParam;
  __shared__ uint32_t smem[8][MEDIUM_BIN];
  BATCH_LOOP(BK_FINALIZE)
    binFinalizeBody(I.T * cfg.tileDepthBins, ts.binCount, ts.binOffset, ts.blockSums, ts.keys, I.segBuf, I.tiles,
                    ts.largeBins, smem, local, nLocal);
  }
}

__global__ void __launch_bounds__(1024) largeBinsBatch(BatchView b, HfbConfig cfgParam) {
  const HfbConfig cfg = cfgParam;
  extern __shared__ uint32_t sk[];
  BATCH_LOOP(BK_LARGE)
    largeBinsBody(ts.largeBins, ts.binCount, ts.binOffset, ts.blockSums, ts.keys, I.segBuf, I.tiles, sk, local,
                  nLocal);
  }
}

__global__ void __launch_bounds__(1024) tileSortBatch(BatchView b, HfbConfig cfgParam) {
  const HfbConfig cfg = cfgParam;
  __shared__ SortShared ss;
  BATCH_LOOP(BK_SORT)
    tileSortBody(I.T, cfg.sortBuckets, cfg.sortBucketSize, I.segCount, I.sortBuckets, I.tileList, ss);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024) fineScheduleBatch(BatchView b, HfbConfig cfgParam, uint32_t grid,
                                                          DeviceCounters* __restrict__ counters) {
  const HfbConfig cfg = cfgParam;
  __shared__ uint32_t warpSums[32];
  __shared__ uint32_t totalRecords;
  BATCH_LOOP(BK_SCHEDULE)
    const FineScratch fs = fineScratchLayout(I.scratch, cfg, I.W, I.H);
    const uint32_t dispMode = I.U.displayMode & 0xffu;
    const bool dbg = dispMode == 4u && ((I.U.displayMode >> 8) & 0xffffu) != 0u;
    fineScheduleBody(I.tileList, I.segCount, I.tiles, I.T, cfg.tileDepthBins, grid, I.maxDrawn, I.S * I.P,
                     dbg ? 0u : 1u, fs, counters, warpSums, totalRecords);
  }
}

// Exclusive prefix of the instances' work items; resets the batch queue.
__global__ void __launch_bounds__(1024) fineItemPrefixBatch(BatchView b, HfbConfig cfgParam) {
  const HfbConfig cfg = cfgParam;
  __shared__ uint32_t warpSums[32];
  const uint32_t n = b.hdr->n;
  uint32_t carry = 0;
  for (uint32_t i0 = 0; i0 < n; i0 += blockDim.x) {
    const uint32_t i = i0 + threadIdx.x;
    uint32_t items = 0;
    if (i < n) {
      const BatchInst& I = b.insts[i];
      items = (*HFB_G(&fineScratchLayout(I.scratch, cfg, I.W, I.H).hdr[0]));
    }
    uint32_t chunk;
    const uint32_t ex = blockExclusiveScan(items, warpSums, chunk);
    if (i < n) b.itemPrefix[i] = carry + ex;
    carry += chunk;
  }
  if (threadIdx.x == 0) {
    b.itemPrefix[n] = carry;
    b.hdr->fineQueue = 0;
  }
}
#undef BATCH_LOOP

template <int TS, int MAXL>
cudaError_t launchFineBatchT(HfbCtx* c, const BatchView& b) {
  HFB_CHECK_BIND(c);
  const HfbConfig& cfg = c->cfg;
  constexpr size_t SMEM = sizeof(FineSmem<TS>);
  uint32_t& grid = c->batchGrid[BK_COUNT];  // the fine kernel's persistent grid
  if (!grid) {
    cudaError_t e = cudaFuncSetAttribute(fineBatch<TS, MAXL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    int per = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fineBatch<TS, MAXL>, TS * TS, SMEM);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorInvalidConfiguration;
    grid = cfg.processorCount ? cfg.processorCount : (uint32_t)per * c->smCount;
  }
  DeviceCounters* dc = (DeviceCounters*)c->dCounters;
  uint32_t& sgrid = c->batchGrid[BK_SCHEDULE];
  if (!sgrid) sgrid = c->smCount;
  fineScheduleBatch<<<batchLaunchGrid(c, sgrid), 1024, 0, c->stream>>>(b, cfg, batchLaunchGrid(c, grid), dc);
  HFB_AFTER_LAUNCH(c, "fineScheduleBatch");
  fineItemPrefixBatch<<<1, 1024, 0, c->stream>>>(b, cfg);
  HFB_AFTER_LAUNCH(c, "fineItemPrefixBatch");
  FineArgs a{};
  a.B = cfg.tileDepthBins;
  a.L = cfg.slicesPerPixel;
  a.SP = cfg.shadingPoints;
  a.CAP = cfg.avgFragmentsPerSlice * cfg.slicesPerPixel * cfg.tileSize * cfg.tileSize;
  a.alphaQuadratic = cfg.alphaQuadratic;
  a.alphaMul = cfg.alphaMultiplier;
  a.counters = dc;
  fineBatch<TS, MAXL><<<batchLaunchGrid(c, grid), TS * TS, SMEM, c->stream>>>(b, a, cfg);
  HFB_AFTER_LAUNCH(c, "fineBatch");
  c->launches += 3;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launchTilesPass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                            const float* tan, const float* depth, uint32_t strandsToRender, HfbRasterBuffers& rb,
                            float4* proj) {
  HFB_CHECK_BIND(c);
  const HfbConfig& cfg = c->cfg;
  const uint32_t W = rb.width, H = rb.height, TS = cfg.tileSize, B = cfg.tileDepthBins;
  const uint32_t T = divCeil(W, TS) * divCeil(H, TS);
  const uint32_t TB = T * B;
  TilesScratch s = tilesScratchLayout(rb.scratch, cfg, W, H, rb.maxDrawnSegments);
  cudaError_t e = cudaMemsetAsync(s.binCount, 0, (size_t)TB * 4, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.largeBins, 0, 4, c->stream);
  if (e != cudaSuccess) return e;
  const uint32_t nStrands = min(strandsToRender, h.strandsCount);
  const uint32_t nSeg = nStrands * (h.pointsPerStrand - 1u);
  DeviceCounters* dc = (DeviceCounters*)c->dCounters;
  if (nSeg) {
    float4 bs = make_float4(h.boundingSphere[0], h.boundingSphere[1], h.boundingSphere[2], h.boundingSphere[3]);
    tilesRasterKernel<<<divCeil(nSeg, TR_SEGS), TR_SEGS, 0, c->stream>>>(
        u, h.pointsPerStrand, nStrands, TS, B, cfg.invalidTilesPerSegmentThreshold, bs, (const float4*)pos,
        (const float4*)tan, depth, (uint4*)rb.tiles, rb.tileSegments, rb.segmentCountPerTile, s.binCount, dc, proj);
    HFB_AFTER_LAUNCH(c, "tilesRasterKernel");
  }
  const uint32_t nBlocks = divCeil(TB, SCAN_PER_BLOCK);
  binScanBlocks<<<nBlocks, 512, 0, c->stream>>>(s.binCount, s.binOffset, s.blockSums, TB);
  HFB_AFTER_LAUNCH(c, "binScanBlocks");
  binScanSums<<<1, 1024, 0, c->stream>>>(s.blockSums, nBlocks);
  HFB_AFTER_LAUNCH(c, "binScanSums");
  binScatterKernel<<<c->smCount * 4, 256, 0, c->stream>>>(rb.tileSegments, rb.maxDrawnSegments, s.binOffset,
                                                          s.blockSums, s.keys, dc, TB);
  HFB_AFTER_LAUNCH(c, "binScatterKernel");
  binFinalizeKernel<<<min(divCeil(TB, 8), (uint32_t)c->smCount * 16), 256, 0, c->stream>>>(
      TB, s.binCount, s.binOffset, s.blockSums, s.keys, rb.tileSegments, (uint4*)rb.tiles, s.largeBins);
  HFB_AFTER_LAUNCH(c, "binFinalizeKernel");
  if (!c->largeBinsAttrSet) {
    e = cudaFuncSetAttribute(largeBinsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, LARGE_SMEM_KEYS * 4);
    if (e != cudaSuccess) return e;
    c->largeBinsAttrSet = true;
  }
  largeBinsKernel<<<c->smCount, 1024, LARGE_SMEM_KEYS * 4, c->stream>>>(
      s.largeBins, s.binCount, s.binOffset, s.blockSums, s.keys, rb.tileSegments, (uint4*)rb.tiles);
  HFB_AFTER_LAUNCH(c, "largeBinsKernel");
  c->launches += nSeg ? 6 : 5;
  return cudaGetLastError();
}

// Loads the tiles pass's kernels onto the current device and sets the
// large-bins kernel's shared-memory attribute.  CUDA loads device code
// lazily, at a kernel's first launch or attribute query, and loading takes
// device memory for the code; hfb_tiles_pass_noalloc's set-up calls this at
// context creation so that its own launches load (allocate) nothing.
cudaError_t tilesPassLoad(HfbCtx* c) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, tilesRasterKernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, binScanBlocks);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, binScanSums);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, binScatterKernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, binFinalizeKernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, largeBinsKernel);
  if (e == cudaSuccess && !c->largeBinsAttrSet) {
    e = cudaFuncSetAttribute(largeBinsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, LARGE_SMEM_KEYS * 4);
    if (e == cudaSuccess) c->largeBinsAttrSet = true;
  }
  return e;
}

cudaError_t launchTileSort(HfbCtx* c, HfbRasterBuffers& rb) {
  HFB_CHECK_BIND(c);
  const HfbConfig& cfg = c->cfg;
  const uint32_t T = divCeil(rb.width, cfg.tileSize) * divCeil(rb.height, cfg.tileSize);
  if (cfg.sortBuckets > SORT_MAX_BUCKETS) return cudaErrorInvalidValue;
  tileSortKernel<<<1, 1024, 0, c->stream>>>(T, cfg.sortBuckets, cfg.sortBucketSize, rb.segmentCountPerTile,
                                            rb.sortBuckets, rb.tileList);
  HFB_AFTER_LAUNCH(c, "tileSortKernel");
  c->launches += 1;
  return cudaGetLastError();
}

cudaError_t launchFinePass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                           const float* tan, const float* shading, const float* depth, HfbRasterBuffers& rb,
                           const float4* proj) {
  const uint32_t TS = c->cfg.tileSize, L = c->cfg.slicesPerPixel;
  if (TS == 8) {
    if (L <= 4) return launchFineT<8, 4>(c, u, h, pos, tan, shading, depth, rb, proj);
    if (L <= 8) return launchFineT<8, 8>(c, u, h, pos, tan, shading, depth, rb, proj);
    return launchFineT<8, 16>(c, u, h, pos, tan, shading, depth, rb, proj);
  }
  if (TS == 16) {
    if (L <= 4) return launchFineT<16, 4>(c, u, h, pos, tan, shading, depth, rb, proj);
    if (L <= 8) return launchFineT<16, 8>(c, u, h, pos, tan, shading, depth, rb, proj);
    return launchFineT<16, 16>(c, u, h, pos, tan, shading, depth, rb, proj);
  }
  if (L <= 4) return launchFineT<32, 4>(c, u, h, pos, tan, shading, depth, rb, proj);
  if (L <= 8) return launchFineT<32, 8>(c, u, h, pos, tan, shading, depth, rb, proj);
  return cudaErrorInvalidValue;  // 32x32 tiles with more than 8 slices: too many registers per pixel
}

}  // namespace hfb

namespace hfb {

cudaError_t launchBatchTiles(HfbCtx* c, const BatchView& b) {
  HFB_CHECK_BIND(c);
  const HfbConfig& cfg = c->cfg;
  DeviceCounters* dc = (DeviceCounters*)c->dCounters;
  uint32_t* g = c->batchGrid;
  if (!g[BK_RASTER]) {
    int per = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tilesRasterBatch, TR_SEGS, 0);
    if (e != cudaSuccess) return e;
    g[BK_RASTER] = (uint32_t)(per > 0 ? per : 1) * c->smCount;
    g[BK_SCAN] = c->smCount * 4u;
    g[BK_SCAN_SUMS] = c->smCount;
    g[BK_SCATTER] = c->smCount * 8u;
    g[BK_FINALIZE] = c->smCount * 8u;
    g[BK_LARGE] = c->smCount * 2u;
    e = cudaFuncSetAttribute(largeBinsBatch, cudaFuncAttributeMaxDynamicSharedMemorySize, LARGE_SMEM_KEYS * 4);
    if (e != cudaSuccess) return e;
  }
  tilesRasterBatch<<<batchLaunchGrid(c, g[BK_RASTER]), TR_SEGS, 0, c->stream>>>(b, cfg, dc);
  HFB_AFTER_LAUNCH(c, "tilesRasterBatch");
  binScanBatch<<<batchLaunchGrid(c, g[BK_SCAN]), 512, 0, c->stream>>>(b, cfg);
  HFB_AFTER_LAUNCH(c, "binScanBatch");
  binScanSumsBatch<<<batchLaunchGrid(c, g[BK_SCAN_SUMS]), 1024, 0, c->stream>>>(b, cfg);
  HFB_AFTER_LAUNCH(c, "binScanSumsBatch");
  binScatterBatch<<<batchLaunchGrid(c, g[BK_SCATTER]), 256, 0, c->stream>>>(b, cfg, dc);
  HFB_AFTER_LAUNCH(c, "binScatterBatch");
  binFinalizeBatch<<<batchLaunchGrid(c, g[BK_FINALIZE]), 256, 0, c->stream>>>(b, cfg);
  HFB_AFTER_LAUNCH(c, "binFinalizeBatch");
  largeBinsBatch<<<batchLaunchGrid(c, g[BK_LARGE]), 1024, LARGE_SMEM_KEYS * 4, c->stream>>>(b, cfg);
  HFB_AFTER_LAUNCH(c, "largeBinsBatch");
  c->launches += 6;
  return cudaGetLastError();
}

cudaError_t launchBatchSort(HfbCtx* c, const BatchView& b) {
  HFB_CHECK_BIND(c);
  if (c->cfg.sortBuckets > SORT_MAX_BUCKETS) return cudaErrorInvalidValue;
  uint32_t& grid = c->batchGrid[BK_SORT];
  if (!grid) grid = c->smCount;
  tileSortBatch<<<batchLaunchGrid(c, grid), 1024, 0, c->stream>>>(b, c->cfg);
  HFB_AFTER_LAUNCH(c, "tileSortBatch");
  c->launches += 1;
  return cudaGetLastError();
}

cudaError_t launchBatchFine(HfbCtx* c, const BatchView& b) {
  const uint32_t TS = c->cfg.tileSize, L = c->cfg.slicesPerPixel;
  if (TS == 8) {
    if (L <= 4) return launchFineBatchT<8, 4>(c, b);
    if (L <= 8) return launchFineBatchT<8, 8>(c, b);
    return launchFineBatchT<8, 16>(c, b);
  }
  if (TS == 16) {
    if (L <= 4) return launchFineBatchT<16, 4>(c, b);
    if (L <= 8) return launchFineBatchT<16, 8>(c, b);
    return launchFineBatchT<16, 16>(c, b);
  }
  if (L <= 4) return launchFineBatchT<32, 4>(c, b);
  if (L <= 8) return launchFineBatchT<32, 8>(c, b);
  return cudaErrorInvalidValue;
}

}  // namespace hfb
