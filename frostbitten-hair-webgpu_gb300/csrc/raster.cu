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
//   4. binFinalize   one warp per (tile, bin): sort its keys ascending and
//                    write the reference's linked list (head -> largest key).
//   5. largeBins     one CTA per bin with more than 1024 records.
// The resulting lists are canonical: they do not depend on atomic order.
#include <cooperative_groups.h>
#include <cuda_fp16.h>

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
  projectHairPoint(U.modelMatrix.m, U.vpMatrix.m, cam, ld4(__ldg(&pos[i])), ld4(__ldg(&tan[i])), size,
                   U.fiberRadius, r.v00, r.v01, r.depthsProj.x, r.depthsProj.y);
  projectHairPoint(U.modelMatrix.m, U.vpMatrix.m, cam, ld4(__ldg(&pos[i + 1])), ld4(__ldg(&tan[i + 1])), size,
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

// ---------------------------------------------------------------------------
// 1. tilesRaster: HairTilesPass.main + processTile, hairTilesPass.wgsl.ts:70-238
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128)
tilesRasterKernel(const HfbUniforms U, uint32_t P, uint32_t nStrands, uint32_t TS, uint32_t B,
                  uint32_t threshold, float4 bsphere, const float4* __restrict__ pos,
                  const float4* __restrict__ tan, const float* __restrict__ depth, uint4* __restrict__ tiles,
                  uint32_t* __restrict__ segBuf, uint32_t* __restrict__ segCount,
                  uint32_t* __restrict__ binCount, DeviceCounters* __restrict__ counters) {
  const uint32_t segsPerStrand = P - 1u;
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nStrands * segsPerStrand) return;
  const uint32_t strand = gid / segsPerStrand, seg = gid - strand * segsPerStrand;
  const f2 size = mk2(U.viewport.x, U.viewport.y);
  const uint32_t W = f2u(size.x), H = f2u(size.y);
  const uint32_t tilesX = divCeil(W, TS);
  const uint32_t maxDrawn = U.maxDrawnHairSegments;

  ProjSeg s = projectSegment(U, pos, tan, P, strand, seg, size);
  // getRasterizedHairBounds, swRasterizeHair.wgsl.ts:111-124
  float bx1 = fminf(ceilf(fmaxf(fmaxf(s.v00.x, s.v01.x), fmaxf(s.v10.x, s.v11.x))), size.x);
  float by1 = fminf(ceilf(fmaxf(fmaxf(s.v00.y, s.v01.y), fmaxf(s.v10.y, s.v11.y))), size.y);
  float bx0 = fmaxf(floorf(fminf(fminf(s.v00.x, s.v01.x), fminf(s.v10.x, s.v11.x))), 0.0f);
  float by0 = fmaxf(floorf(fminf(fminf(s.v00.y, s.v01.y), fminf(s.v10.y, s.v11.y))), 0.0f);
  const uint32_t ux0 = f2u(bx0), uy0 = f2u(by0), ux1 = f2u(bx1), uy1 = f2u(by1);
  const uint32_t tminx = ux0 / TS, tminy = uy0 / TS, tmaxx = ux1 / TS, tmaxy = uy1 / TS;
  const uint32_t tsx = (tmaxx - tminx) + 1u, tsy = (tmaxy - tminy) + 1u;
  if (tsx * tsy > threshold) return;  // degenerate segment rejection, :111-117

  // getHairDepthBoundsVS, :242-246
  f4 bsVS = m4v(U.modelViewMat.m, mk4(bsphere.x, bsphere.y, bsphere.z, 1.0f));
  const float dv0 = fsub(bsVS.z, bsphere.w), dv1 = fadd(bsVS.z, bsphere.w);
  const uint32_t key = (strand << 8) | seg;

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
          f3 vs = projectVertex(U.projMatrixInv.m, mk4(p.x, p.y, hd, 1.0f));
          uint32_t bin = (B - 1u) - getDepthBin(B, dv0, dv1, vs.z);
          dmin = fminf(dmin, hd);
          dmax = fmaxf(dmax, hd);
          dbin = min(dbin, bin);
        }
      }
      if (dmin > 1.0f) continue;
      // store the result, :220-237 (warp-aggregated pointer allocation)
      cg::coalesced_group g = cg::coalesced_threads();
      uint32_t base = 0;
      if (g.thread_rank() == 0) base = atomicAdd(&segBuf[0], g.size());
      base = g.shfl(base, 0);
      uint32_t ptr = base + g.thread_rank();
      if (ptr < maxDrawn) {
        uint32_t ti = ty * tilesX * B + tx * B + dbin;
        // _storeTileHead: min / max depth as u32 maxima (order independent)
        atomicMax(&tiles[ti].x, f2u(fmul(fsub(1.0f, dmin), F_MAX_U32)));
        atomicMax(&tiles[ti].y, f2u(fmul(dmax, F_MAX_U32)));
        atomicAdd(&segCount[ty * tilesX + tx], 1u);  // _incTileSegmentCount
        atomicAdd(&binCount[ti], 1u);
        // staging record in the list slot; binFinalize rewrites it
        segBuf[1u + 2u * ptr] = ti;
        segBuf[2u + 2u * ptr] = key;
      } else {
        atomicAdd(&counters->tileRecordsDropped, 1ull);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 2. binScan: exclusive prefix over T*B counts (block-local + block sums)
// ---------------------------------------------------------------------------
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

__global__ void __launch_bounds__(512) binScanBlocks(const uint32_t* __restrict__ cnt, uint32_t* __restrict__ off,
                                                     uint32_t* __restrict__ blockSums, uint32_t n) {
  __shared__ uint32_t warpSums[32];
  const uint32_t base = blockIdx.x * SCAN_PER_BLOCK + threadIdx.x * 4u;
  uint32_t v[4], s = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[k] = base + k < n ? cnt[base + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t ex = blockExclusiveScan(s, warpSums, total);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (base + k < n) off[base + k] = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) binScanSums(uint32_t* __restrict__ blockSums, uint32_t nBlocks) {
  __shared__ uint32_t warpSums[32];
  uint32_t carry = 0;
  for (uint32_t b0 = 0; b0 < nBlocks; b0 += blockDim.x) {
    uint32_t i = b0 + threadIdx.x;
    uint32_t v = i < nBlocks ? blockSums[i] : 0u;
    uint32_t total;
    uint32_t ex = blockExclusiveScan(v, warpSums, total);
    if (i < nBlocks) blockSums[i] = carry + ex;
    carry += total;
  }
}

// ---------------------------------------------------------------------------
// 3. binScatter: keys into CSR order (order inside a bin fixed by step 4)
// ---------------------------------------------------------------------------
__global__ void binScatterKernel(const uint32_t* __restrict__ segBuf, uint32_t maxDrawn,
                                 uint32_t* __restrict__ binOffset, const uint32_t* __restrict__ blockSums,
                                 uint32_t* __restrict__ keys, DeviceCounters* __restrict__ counters) {
  const uint32_t total = segBuf[0];
  const uint32_t n = min(total, maxDrawn);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&counters->tileRecords, (unsigned long long)total);
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    uint32_t ti = segBuf[1u + 2u * r];
    uint32_t key = segBuf[2u + 2u * r];
    uint32_t pos = blockSums[ti / SCAN_PER_BLOCK] + atomicAdd(&binOffset[ti], 1u);
    keys[pos] = key;
  }
}

// ---------------------------------------------------------------------------
// 4. binFinalize: per-bin sort + reference linked list (warp per bin)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void writeList(uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles, uint32_t ti,
                                          uint32_t start, uint32_t i, uint32_t n, uint32_t key) {
  // _storeTileSegment encoding: (segment << 24) | strand; next = previous
  // (smaller) key, so the walk from the head visits keys in descending order.
  uint32_t p = start + i;
  segBuf[1u + 2u * p] = ((key & 0xffu) << 24) | (key >> 8);
  segBuf[2u + 2u * p] = i == 0 ? INVALID_PTR : p - 1u;
  if (i == n - 1u) {
    tiles[ti].z = p + 1u;  // head pointer (+1, 0 = empty)
    tiles[ti].w = n;       // padding0: list length, a hint the fine pass verifies
  }
}

__global__ void __launch_bounds__(256)
binFinalizeKernel(uint32_t TB, const uint32_t* __restrict__ binCount, const uint32_t* __restrict__ binOffset,
                  const uint32_t* __restrict__ blockSums, uint32_t* __restrict__ keys,
                  uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles, uint32_t* __restrict__ largeBins) {
  __shared__ uint32_t smem[8][MEDIUM_BIN];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  uint32_t* s = smem[warp];
  for (uint32_t ti = gw; ti < TB; ti += nw) {
    const uint32_t n = binCount[ti];
    if (n == 0) continue;
    const uint32_t end = blockSums[ti / SCAN_PER_BLOCK] + binOffset[ti];  // cursor ended at bin end
    const uint32_t start = end - n;
    if (n <= SMALL_BIN) {
      uint32_t v = lane < n ? keys[start + lane] : 0xffffffffu;
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
      for (uint32_t i = lane; i < N; i += 32) s[i] = i < n ? keys[start + i] : 0xffffffffu;
      __syncwarp();
      for (uint32_t k = 2; k <= N; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
          for (uint32_t c = lane; c < N / 2; c += 32) {
            uint32_t a = 2u * j * (c / j) + (c % j), b = a + j;
            uint32_t x = s[a], y = s[b];
            bool asc = (a & k) == 0;
            if ((x > y) == asc) { s[a] = y; s[b] = x; }
          }
          __syncwarp();
        }
      }
      for (uint32_t i = lane; i < n; i += 32) writeList(segBuf, tiles, ti, start, i, n, s[i]);
      __syncwarp();
    } else if (lane == 0) {
      uint32_t slot = atomicAdd(&largeBins[0], 1u);
      largeBins[1u + slot] = ti;
    }
  }
}

// ---------------------------------------------------------------------------
// 5. largeBins: one CTA per bin with > MEDIUM_BIN records.  Runs of
//    LARGE_SMEM_KEYS are bitonic-sorted in shared memory, then merged pairwise
//    through the bin's own list slots (free until the final write) by rank
//    search (keys are unique).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024)
largeBinsKernel(const uint32_t* __restrict__ largeBins, const uint32_t* __restrict__ binCount,
                const uint32_t* __restrict__ binOffset, const uint32_t* __restrict__ blockSums,
                uint32_t* __restrict__ keys, uint32_t* __restrict__ segBuf, uint4* __restrict__ tiles) {
  extern __shared__ uint32_t sk[];
  const uint32_t nLarge = largeBins[0];
  for (uint32_t li = blockIdx.x; li < nLarge; li += gridDim.x) {
    const uint32_t ti = largeBins[1u + li];
    const uint32_t n = binCount[ti];
    const uint32_t start = blockSums[ti / SCAN_PER_BLOCK] + binOffset[ti] - n;
    uint32_t* a = keys + start;
    uint32_t* tmp = segBuf + 1u + 2u * start;  // 2n free words
    // sort runs in shared memory
    for (uint32_t r0 = 0; r0 < n; r0 += LARGE_SMEM_KEYS) {
      uint32_t m = min(LARGE_SMEM_KEYS, n - r0);
      uint32_t N = 2;
      while (N < m) N <<= 1;
      for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) sk[i] = i < m ? a[r0 + i] : 0xffffffffu;
      __syncthreads();
      for (uint32_t k = 2; k <= N; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
          for (uint32_t c = threadIdx.x; c < N / 2; c += blockDim.x) {
            uint32_t x0 = 2u * j * (c / j) + (c % j), x1 = x0 + j;
            uint32_t x = sk[x0], y = sk[x1];
            bool asc = (x0 & k) == 0;
            if ((x > y) == asc) { sk[x0] = y; sk[x1] = x; }
          }
          __syncthreads();
        }
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) a[r0 + i] = sk[i];
      __syncthreads();
    }
    // merge passes (ping-pong between a and tmp)
    uint32_t* src = a;
    uint32_t* dst = tmp;
    for (uint32_t run = LARGE_SMEM_KEYS; run < n; run <<= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t blk = i / (2u * run);
        uint32_t l0 = blk * 2u * run, l1 = min(l0 + run, n), r1 = min(l0 + 2u * run, n);
        uint32_t v = src[i];
        bool left = i < l1;
        uint32_t o0 = left ? l1 : l0, o1 = left ? r1 : l1;  // the other run
        uint32_t lo = o0, hi = o1;                           // count of other < v
        while (lo < hi) {
          uint32_t mid = (lo + hi) >> 1;
          if (src[mid] < v) lo = mid + 1; else hi = mid;
        }
        uint32_t rankOther = lo - o0;
        uint32_t rankSelf = i - (left ? l0 : l1);
        dst[l0 + rankSelf + rankOther] = v;
      }
      __syncthreads();
      uint32_t* t = src; src = dst; dst = t;
    }
    if (src != a) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) a[i] = src[i];
      __syncthreads();
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) writeList(segBuf, tiles, ti, start, i, n, a[i]);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// HairTileSortPass (count-tiles + sort) in one CTA, stable inside a bucket.
// ---------------------------------------------------------------------------
constexpr uint32_t SORT_MAX_BUCKETS = 256;

__global__ void __launch_bounds__(1024)
tileSortKernel(uint32_t T, uint32_t NB, uint32_t bucketSize, const uint32_t* __restrict__ segCount,
               uint32_t* __restrict__ buckets, uint32_t* __restrict__ tileList) {
  __shared__ uint32_t hist[SORT_MAX_BUCKETS], offs[SORT_MAX_BUCKETS], run[SORT_MAX_BUCKETS];
  __shared__ uint32_t wcnt[32][SORT_MAX_BUCKETS];
  __shared__ uint32_t drawn;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  for (uint32_t b = tid; b < NB; b += blockDim.x) { hist[b] = 0; run[b] = 0; }
  if (tid == 0) drawn = 0;
  __syncthreads();
  // count-tiles: calcTileSortBucket, hairTileSortPass.countTiles.wgsl.ts:37-40
  uint32_t local = 0;
  for (uint32_t t = tid; t < T; t += blockDim.x) {
    uint32_t c = segCount[t];
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
    buckets[2u * b] = hist[b];
    buckets[2u * b + 1u] = hist[b];  // the in-bucket write counter ends at tileCount
  }
  if (tid == 0) tileList[0] = drawn;
  __syncthreads();
  // stable scatter, one 1024-tile chunk at a time
  for (uint32_t c0 = 0; c0 < T; c0 += blockDim.x) {
    for (uint32_t i = tid; i < 32u * NB; i += blockDim.x) wcnt[i / NB][i % NB] = 0;
    __syncthreads();
    uint32_t t = c0 + tid;
    uint32_t c = t < T ? segCount[t] : 0u;
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
    if (valid) tileList[1u + offs[b] + wcnt[warp][b] + rank] = t;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// HairFinePass: persistent CTAs, one thread per tile pixel.
//
// Per depth bin, the bin's list is walked in chunks of 32 segments (a warp
// reads the list speculatively as a contiguous run and falls back to pointer
// chasing where it is not), the chunk is projected in parallel into shared
// memory, and every pixel tests the chunk in list order.  Each slice of a
// pixel keeps the closed form of its front-to-back blend in registers:
// fragments arrive back to front (descending key) and acc = f + (1 - f.a) *
// acc, which equals the reference's per-slice linked list reduced front to
// back (reduceHairSlices.wgsl.ts:9-73) -- no fragment pool in memory.  The
// fragment-pool capacity of the reference (SLICE_DATA_PER_PROCESSOR_COUNT,
// processHairSegment.wgsl.ts:33-40, hairFinePass.wgsl.ts:258-264) is kept
// exactly: slots are counted per segment in pixel order and the list walk
// stops after the segment that fills the pool.
// ---------------------------------------------------------------------------
constexpr uint32_t CHUNK = 32;     // segments per exact-path sub-chunk (32-bit masks)
constexpr uint32_t STAGE = 256;    // segments staged in shared memory per round
constexpr uint32_t NSHADE = 4;     // shading entries staged per segment

struct FineShared {
  ProjSeg seg[STAGE];
  float4 shade[STAGE][NSHADE];  // the shading entries each segment can sample
  uint32_t strand[STAGE];
  uint32_t segIdx[STAGE];
  uint32_t box[STAGE];       // tile-local pixel-corner bbox x0|y0<<8|x1<<16|y1<<24 (x0 > x1: empty)
  uint32_t area[STAGE];      // pixels of the bbox (upper bound of the segment's fragments)
  uint32_t shadeBase[STAGE]; // first staged shading index | count << 16
  uint4 head[64];            // the tile's HairTileResult per depth bin
  uint32_t binOff[65];       // whole-tile staging: first staged segment of each bin
  uint32_t cnt[32][CHUNK];   // per-warp passing counts per segment (exact path)
  uint32_t red[32];
  uint32_t n, nextPtr, queueIdx, bad, tileMode, total;
  uint32_t cutSeg, cutSlots, chunkTotal;
};

__device__ __forceinline__ bool inBox(uint32_t box, uint32_t lx, uint32_t ly) {
  return lx >= (box & 0xffu) && ly >= ((box >> 8) & 0xffu) && lx <= ((box >> 16) & 0xffu) && ly <= (box >> 24);
}

// edge + depth test of processHairSegment (:5-31); fills w / hd when it passes
__device__ __forceinline__ bool fragmentPasses(const ProjSeg& s, f2 pp, float zbuf, f2& w, float& hd) {
  if (!insideQuad(s, pp)) return false;
  w = interpolateHairQuad(s, pp);
  hd = interpolateHairF32(w, s.depthsProj);
  return hd < zbuf;  // depth test with GL_LESS (skip when >=)
}

// Colour of one fragment (processHairSegment.wgsl.ts:43-53), rounded through
// f16 like pack2x16float (hairSlicesDataBuffer.ts:50-63), blended in front of
// the slice's accumulated colour.  The two shading entries come from the
// segment's staged copy (or global memory when outside it).
template <int MAXL>
__device__ __forceinline__ void addFragment(f4 (&acc)[MAXL], const FineShared& sh, uint32_t k, f2 w, float hd,
                                            uint32_t P, uint32_t SP, uint32_t L, float td0, float td1,
                                            uint32_t alphaQuadratic, float alphaMul,
                                            const float4* __restrict__ shading) {
  // getAlphaCoverage, processHairSegment.wgsl.ts:60-69
  float alpha = fsub(1.0f, fabsf(fsub(fmul(w.x, 2.0f), 1.0f)));
  if (alphaQuadratic) alpha = sqrtf(alpha);
  alpha = sat(fmul(alpha, alphaMul));
  float tFull = fadd((float)sh.segIdx[k], w.y) / (float)(P - 1u);
  // _sampleShading, hairShadingBuffer.ts:28-38
  uint32_t i0, i1;
  float fr = remapToIndices(SP, tFull, i0, i1);
  const uint32_t e0 = sh.shadeBase[k] & 0xffffu, ne = sh.shadeBase[k] >> 16;
  float4 c0, c1;
  if (i0 - e0 < ne && i1 - e0 < ne) {
    c0 = sh.shade[k][i0 - e0];
    c1 = sh.shade[k][i1 - e0];
  } else {
    const size_t sb = (size_t)sh.strand[k] * SP;
    c0 = __ldg(&shading[sb + i0]);
    c1 = __ldg(&shading[sb + i1]);
  }
  f4 c = mix4(ld4(c0), ld4(c1), fr);
  c.w = fmul(c.w, alpha);
  uint32_t sl = getDepthBin(L, td0, td1, hd);  // getSliceIdx
  f4 q = mk4(__half2float(__float2half_rn(c.x)), __half2float(__float2half_rn(c.y)),
             __half2float(__float2half_rn(c.z)), __half2float(__float2half_rn(c.w)));
  float kk = fsub(1.0f, q.w);
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

// Projects staged segment k, its tile-local bounding box, and stages the
// shading entries its fragments can sample (tFull is monotonic in the
// segment coordinate, so they are [i0(t = 0), i1(t = 1)]).
template <int TS>
__device__ __forceinline__ void projectStaged(const HfbUniforms& U, const float4* __restrict__ pos,
                                              const float4* __restrict__ tan, const float4* __restrict__ shading,
                                              uint32_t S, uint32_t P, uint32_t SP, f2 size, uint32_t x0,
                                              uint32_t y0, FineShared& sh, uint32_t k) {
  const uint32_t st = sh.strand[k], sg = sh.segIdx[k];
  ProjSeg s;
  uint32_t box = 0x00ff00ffu, area = 0, shadeBase = 0;  // empty
  if (st < S && sg + 1u < P) {
    s = projectSegment(U, pos, tan, P, st, sg, size);
    // pixel corners that can pass the edge tests: [floor(min), ceil(max)]
    float mnx = floorf(fminf(fminf(s.v00.x, s.v01.x), fminf(s.v10.x, s.v11.x))) - (float)x0;
    float mny = floorf(fminf(fminf(s.v00.y, s.v01.y), fminf(s.v10.y, s.v11.y))) - (float)y0;
    float mxx = ceilf(fmaxf(fmaxf(s.v00.x, s.v01.x), fmaxf(s.v10.x, s.v11.x))) - (float)x0;
    float mxy = ceilf(fmaxf(fmaxf(s.v00.y, s.v01.y), fmaxf(s.v10.y, s.v11.y))) - (float)y0;
    if (mnx <= mxx && mny <= mxy && mxx >= 0.0f && mxy >= 0.0f && mnx <= (float)(TS - 1) && mny <= (float)(TS - 1)) {
      uint32_t bx0 = (uint32_t)fmaxf(mnx, 0.0f), by0 = (uint32_t)fmaxf(mny, 0.0f);
      uint32_t bx1 = (uint32_t)fminf(mxx, (float)(TS - 1)), by1 = (uint32_t)fminf(mxy, (float)(TS - 1));
      box = bx0 | (by0 << 8) | (bx1 << 16) | (by1 << 24);
      area = (bx1 - bx0 + 1u) * (by1 - by0 + 1u);
      uint32_t a0, a1, b0, b1;
      remapToIndices(SP, fadd((float)sg, 0.0f) / (float)(P - 1u), a0, a1);
      remapToIndices(SP, fadd((float)sg, 1.0f) / (float)(P - 1u), b0, b1);
      const uint32_t ne = min(b1 - a0 + 1u, NSHADE);
      const size_t sb = (size_t)st * SP;
      for (uint32_t e = 0; e < ne; e++) sh.shade[k][e] = __ldg(&shading[sb + a0 + e]);
      shadeBase = a0 | (ne << 16);
    }
  } else {  // not a segment of this hair: covers no pixel
    const float nan = __int_as_float(0x7fffffff);
    s.v00 = s.v01 = s.v10 = s.v11 = mk2(nan, nan);
    s.depthsProj = mk4(nan, nan, nan, nan);
  }
  sh.seg[k] = s;
  sh.box[k] = box;
  sh.area[k] = area;
  sh.shadeBase[k] = shadeBase;
}

// Block-wide sum (all threads call; every thread gets the total).
template <int NW>
__device__ __forceinline__ uint32_t blockSum(uint32_t v, FineShared& sh, uint32_t lane, uint32_t warp) {
  const uint32_t w = __reduce_add_sync(0xffffffffu, v);
  if (lane == 0) sh.red[warp] = w;
  __syncthreads();
  uint32_t t = 0;
#pragma unroll
  for (int i = 0; i < NW; i++) t += sh.red[i];
  __syncthreads();
  return t;
}

// Per-bin state of one pixel and of the whole tile (uniform members).
template <int MAXL>
struct BinState {
  f4 acc[MAXL];
  uint32_t nFrag, pending;            // per pixel
  uint32_t running, runningUB;        // uniform: slots allocated (exact / upper bound)
  bool stop;                          // uniform: the pool filled
};

// Rasterizes staged segments [s0, s0 + n) of the current bin in list order
// (processHairSegment for every pixel), keeping the reference's fragment
// pool accounting exact.  Called by every thread of the CTA.
template <int TS, int MAXL>
__device__ __forceinline__ void rasterRange(BinState<MAXL>& st, FineShared& sh, uint32_t s0, uint32_t n,
                                            uint32_t active, uint32_t CAP, bool done, f2 pp, float zbuf,
                                            uint32_t lx, uint32_t ly, uint32_t lane, uint32_t warp, uint32_t tid,
                                            uint32_t P, uint32_t SP, uint32_t L, float td0, float td1,
                                            uint32_t alphaQuadratic, float alphaMul,
                                            const float4* __restrict__ shading,
                                            DeviceCounters* __restrict__ counters) {
  constexpr int NW = TS * TS / 32;
  for (uint32_t c0 = s0; c0 < s0 + n && !st.stop; c0 += CHUNK) {
    const uint32_t cn = min(CHUNK, s0 + n - c0);
    uint32_t bound = 0;
    for (uint32_t j = 0; j < cn; j++) bound += min(sh.area[c0 + j], active);
    if (st.runningUB + bound > CAP) {  // tighten: exact count of what was added so far
      st.running += blockSum<NW>(st.pending, sh, lane, warp);
      st.pending = 0;
      st.runningUB = st.running;
    }
    if (st.runningUB + bound <= CAP) {
      // ---- fast path: the pool cannot fill inside this sub-chunk ----
      if (!done) {
        for (uint32_t j = c0; j < c0 + cn; j++) {
          if (!inBox(sh.box[j], lx, ly)) continue;
          f2 w; float hd;
          if (!fragmentPasses(sh.seg[j], pp, zbuf, w, hd)) continue;
          st.pending++;
          st.nFrag++;
          addFragment<MAXL>(st.acc, sh, j, w, hd, P, SP, L, td0, td1, alphaQuadratic, alphaMul, shading);
        }
      }
      st.runningUB += bound;
    } else {
      // ---- exact path: slots in pixel order, stop at the filling segment ----
      uint32_t mask = 0;
      if (!done) {
        for (uint32_t j = 0; j < cn; j++) {
          if (!inBox(sh.box[c0 + j], lx, ly)) continue;
          f2 w; float hd;
          if (fragmentPasses(sh.seg[c0 + j], pp, zbuf, w, hd)) mask |= 1u << j;
        }
      }
      for (uint32_t j = 0; j < cn; j++) {
        const uint32_t bal = __ballot_sync(0xffffffffu, (mask >> j) & 1u);
        if (lane == 0) sh.cnt[warp][j] = __popc(bal);
      }
      __syncthreads();
      if (warp == 0) {
        uint32_t c = 0;
        if (lane < cn)
          for (int w2 = 0; w2 < NW; w2++) c += sh.cnt[w2][lane];
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t fb = __ballot_sync(0xffffffffu, lane < cn && st.running + incl >= CAP);
        const uint32_t j = fb ? (uint32_t)(__ffs(fb) - 1) : 0u;
        const uint32_t exclJ = __shfl_sync(0xffffffffu, incl - c, j);
        const uint32_t total = __shfl_sync(0xffffffffu, incl, cn - 1u);
        if (lane == 0) {
          sh.cutSeg = fb ? j : CHUNK;
          sh.cutSlots = fb ? CAP - (st.running + exclJ) : 0u;
          sh.chunkTotal = total;
        }
      }
      __syncthreads();
      const uint32_t cutSeg = sh.cutSeg, cutSlots = sh.cutSlots;
      uint32_t m = mask;
      if (cutSeg < CHUNK) {
        uint32_t rank = 0;  // slots taken in the cut segment by lower pixels
        for (uint32_t w2 = 0; w2 < warp; w2++) rank += sh.cnt[w2][cutSeg];
        rank += __popc(__ballot_sync(0xffffffffu, (mask >> cutSeg) & 1u) & ((1u << lane) - 1u));
        m &= cutSeg == 31u ? 0xffffffffu : ((2u << cutSeg) - 1u);  // segments <= cut
        if (rank >= cutSlots) m &= ~(1u << cutSeg);
      }
      while (m) {
        const uint32_t j = __ffs(m) - 1u;
        m &= m - 1u;
        f2 w; float hd;
        fragmentPasses(sh.seg[c0 + j], pp, zbuf, w, hd);
        addFragment<MAXL>(st.acc, sh, c0 + j, w, hd, P, SP, L, td0, td1, alphaQuadratic, alphaMul, shading);
        st.nFrag++;
      }
      st.running = cutSeg < CHUNK ? CAP : st.running + sh.chunkTotal;
      st.runningUB = st.running;
      if (st.running >= CAP) {
        if (tid == 0) atomicAdd(&counters->finePoolFullBins, 1ull);
        st.stop = true;  // the reference breaks after the filling segment
      }
      __syncthreads();  // sh.cnt / cut words are reused
    }
  }
}

template <int TS, int MAXL>
__global__ void __launch_bounds__(TS * TS, TS == 16 ? (MAXL <= 4 ? 3 : 2) : 1)
fineKernel(const HfbUniforms U, uint32_t S, uint32_t P, uint32_t B, uint32_t L, uint32_t SP, uint32_t CAP,
           uint32_t alphaQuadratic, float alphaMul, const float4* __restrict__ pos, const float4* __restrict__ tan,
           const float4* __restrict__ shading, const float* __restrict__ depth, const uint4* __restrict__ tiles,
           const uint32_t* __restrict__ segBuf, const uint32_t* __restrict__ tileList,
           float* __restrict__ result, DeviceCounters* __restrict__ counters) {
  constexpr uint32_t NPX = TS * TS;
  __shared__ FineShared sh;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t lx = tid % TS, ly = tid / TS;
  const f2 size = mk2(U.viewport.x, U.viewport.y);
  const uint32_t W = f2u(size.x), H = f2u(size.y);
  const uint32_t tilesX = divCeil(W, TS), tileCount = tilesX * divCeil(H, TS);
  const uint32_t maxDrawn = U.maxDrawnHairSegments;
  const uint32_t maxProcessed = S * P;  // MAX_PROCESSED_SEGMENTS, hairFinePass.wgsl.ts:212
  const uint32_t dispMode = U.displayMode & 0xffu;
  const uint32_t dbgMax = dispMode == 4u ? ((U.displayMode >> 8) & 0xffffu) : 0u;  // getDbgSlicesModeMaxSlices
  const bool isDbg = dbgMax != 0u;
  const uint32_t drawnTiles = tileList[0];
  // the list array sits at byte offset 4 (hairTileSegmentsBuffer.ts:60-68):
  // only 4-byte loads are aligned there
  uint32_t* queue = reinterpret_cast<uint32_t*>(result);  // tileQueueAtomicIdx
  float4* res = reinterpret_cast<float4*>(result + 4);

  while (true) {
    if (tid == 0) sh.queueIdx = atomicAdd(queue, 1u);  // getNextTileIdx, :294-303
    __syncthreads();
    const uint32_t q = sh.queueIdx;
    if (q >= drawnTiles) break;
    const uint32_t tileIdx = tileList[1u + q];
    if (tileIdx >= tileCount) { __syncthreads(); continue; }
    const uint32_t tx = tileIdx % tilesX, ty = tileIdx / tilesX;
    const TileB tbp = tileBoundsPx(W, H, TS, tx, ty);
    const uint32_t px = tbp.x0 + lx, py = tbp.y0 + ly;
    // Pixels of a partial edge tile outside the viewport take no part.
    const bool inView = px < W && py < H;
    const f2 pp = mk2((float)px, (float)py);
    const float zbuf = inView ? loadTex2DClamp(depth, W, H, f2i(pp.x), f2i(fsub(size.y, pp.y))) : 0.0f;
    bool done = !inView;
    f4 fin = mk4(0.f, 0.f, 0.f, 0.f);  // rasterizerResult was cleared before the pass
    if (tid < B) sh.head[tid] = tiles[ty * tilesX * B + tx * B + tid];
    __syncthreads();

    // ---- whole-tile staging: every bin's list at once when the lists carry
    // a length hint (padding0, written by the tiles pass) that checks out ----
    if (warp == 0) {
      uint32_t ok = 1, sum = 0;
      for (uint32_t b0 = 0; b0 < B; b0 += 32) {
        const uint32_t bb = b0 + lane;
        uint32_t nb = 0;
        if (bb < B) {
          const uint4 h = sh.head[bb];
          const bool nonEmpty = (float)h.y / F_MAX_U32 != 0.0f && h.z != 0u;
          if (nonEmpty) {
            if (h.w != 0u && h.w <= h.z && h.z <= maxDrawn) nb = h.w; else ok = 0;
          }
        }
        uint32_t incl = nb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= (uint32_t)o) incl += y;
        }
        if (bb < B) sh.binOff[bb] = sum + incl - nb;
        sum += __shfl_sync(0xffffffffu, incl, 31);
      }
      ok = __all_sync(0xffffffffu, ok);
      if (lane == 0) {
        sh.binOff[B] = sum;
        sh.total = sum;
        sh.tileMode = ok && sum <= STAGE && sum <= maxProcessed;
        sh.bad = 0;
      }
    }
    __syncthreads();
    bool tileMode = sh.tileMode != 0u;
    if (tileMode) {
      const uint32_t total = sh.total;
      for (uint32_t k = tid; k < total; k += NPX) {
        uint32_t lo = 0, hi = B;  // bin of k: binOff[lo] <= k < binOff[lo + 1]
        while (hi - lo > 1u) {
          const uint32_t mid = (lo + hi) >> 1;
          if (sh.binOff[mid] <= k) lo = mid; else hi = mid;
        }
        const uint4 h = sh.head[lo];
        const uint32_t j = k - sh.binOff[lo];
        const uint32_t idx = h.z - 1u - j;
        const uint32_t enc = __ldg(&segBuf[1u + 2u * idx]);
        const uint32_t nxt = __ldg(&segBuf[2u + 2u * idx]);
        if (nxt != ((j + 1u == h.w) ? INVALID_PTR : idx - 1u)) sh.bad = 1;
        sh.strand[k] = enc & 0x00ffffffu;
        sh.segIdx[k] = enc >> 24;
      }
      __syncthreads();
      tileMode = sh.bad == 0u;
      if (tileMode) {
        for (uint32_t k = tid; k < total; k += NPX)
          projectStaged<TS>(U, pos, tan, shading, S, P, SP, size, tbp.x0, tbp.y0, sh, k);
      }
      __syncthreads();
    }

    for (uint32_t bin = 0; bin < B; bin++) {
      const uint4 head = sh.head[bin];
      // _getTileDepth, hairTilesResultBuffer.ts:47-54
      const float td0 = (float)(0xffffffffu - head.x) / F_MAX_U32;
      const float td1 = (float)head.y / F_MAX_U32;
      if (td1 != 0.0f) {  // processTile, :205-288
        BinState<MAXL> st;
#pragma unroll
        for (int si = 0; si < MAXL; si++) st.acc[si] = mk4(0.f, 0.f, 0.f, 0.f);
        st.nFrag = 0; st.pending = 0; st.running = 0; st.runningUB = 0; st.stop = false;
        const uint32_t active = __syncthreads_count(!done);
        if (tileMode) {
          const uint32_t s0 = sh.binOff[bin], n = sh.binOff[bin + 1] - s0;
          rasterRange<TS, MAXL>(st, sh, s0, n, active, CAP, done, pp, zbuf, lx, ly, lane, warp, tid, P, SP, L,
                                td0, td1, alphaQuadratic, alphaMul, shading, counters);
        } else {
          // ---- per-bin staging: runs of the list (hinted contiguous runs in
          // parallel, otherwise a warp walks it) ----
          uint32_t ptr = head.z == 0u ? INVALID_PTR : head.z - 1u;
          uint32_t hint = (head.w != 0u && head.w <= head.z && head.z <= maxDrawn) ? head.w : 0u;
          uint32_t processed = 0;
          while (!st.stop && ptr != INVALID_PTR && ptr < maxDrawn && processed < maxProcessed) {
            uint32_t n = 0;
            if (hint) {
              n = min(min(hint, STAGE), maxProcessed - processed);
              if (tid == 0) sh.bad = 0;
              __syncthreads();
              for (uint32_t k = tid; k < n; k += NPX) {
                const uint32_t idx = ptr - k;
                const uint32_t enc = __ldg(&segBuf[1u + 2u * idx]);
                const uint32_t nxt = __ldg(&segBuf[2u + 2u * idx]);
                if (nxt != ((k + 1u == hint) ? INVALID_PTR : idx - 1u)) sh.bad = 1;
                sh.strand[k] = enc & 0x00ffffffu;
                sh.segIdx[k] = enc >> 24;
              }
              __syncthreads();
              if (sh.bad) {
                hint = 0;  // not the contiguous layout: walk it
                continue;
              }
              if (tid == 0) sh.nextPtr = (n == hint) ? INVALID_PTR : ptr - n;
              hint -= n;
            } else {
              if (warp == 0) {  // speculative contiguous runs, else pointer chasing
                uint32_t p = ptr, m = 0;
                while (m < CHUNK && p != INVALID_PTR && p < maxDrawn && processed + m < maxProcessed) {
                  const uint32_t want = min(CHUNK - m, maxProcessed - processed - m);
                  const uint32_t cand = p - lane;
                  const bool inRange = lane < want && lane <= p;
                  uint2 e = make_uint2(0u, INVALID_PTR);
                  if (inRange) {
                    e.x = __ldg(&segBuf[1u + 2u * cand]);
                    e.y = __ldg(&segBuf[2u + 2u * cand]);
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
                  }
                  m += cnt;
                  p = firstIn ? firstNext : p - cnt;
                }
                if (lane == 0) { sh.n = m; sh.nextPtr = p; }
              }
              __syncthreads();
              n = sh.n;
            }
            if (n == 0) break;
            for (uint32_t k = tid; k < n; k += NPX)
              projectStaged<TS>(U, pos, tan, shading, S, P, SP, size, tbp.x0, tbp.y0, sh, k);
            __syncthreads();
            const uint32_t nextPtr = sh.nextPtr;
            rasterRange<TS, MAXL>(st, sh, 0, n, active, CAP, done, pp, zbuf, lx, ly, lane, warp, tid, P, SP, L,
                                  td0, td1, alphaQuadratic, alphaMul, shading, counters);
            processed += n;
            __syncthreads();  // the staged run is refilled next iteration
            ptr = nextPtr;
          }
        }
        // reduceHairSlices (runs for every non-empty bin, as in the reference)
        if (!done) {
          if (isDbg) {
            const uint32_t cntAll = f2u(fmul(fin.x, (float)dbgMax)) + st.nFrag;
            fin = mk4(sat((float)cntAll / (float)dbgMax), 0.0f, 0.0f, 1.0f);
          } else {
#pragma unroll
            for (int si = 0; si < MAXL; si++) {
              if ((uint32_t)si < L && fin.w < 0.999f) {
                const float k = fsub(1.0f, fin.w);
                fin.x = fadd(fin.x, fmul(st.acc[si].x, k));
                fin.y = fadd(fin.y, fmul(st.acc[si].y, k));
                fin.z = fadd(fin.z, fmul(st.acc[si].z, k));
                fin.w = fadd(fin.w, fmul(st.acc[si].w, k));
              }
            }
            done = fin.w >= 0.999f;  // isPixelDone with ALPHA_CUTOFF
          }
        }
      }
      // checkAllPixelsInWkgrpDone, :305-327
      if (__syncthreads_and(done)) break;
    }
    if (inView) res[(size_t)py * W + px] = make_float4(fin.x, fin.y, fin.z, fin.w);
    __syncthreads();  // the tile's shared state is rewritten for the next tile
  }
}

template <int TS, int MAXL>
cudaError_t launchFineT(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                        const float* tan, const float* shading, const float* depth, HfbRasterBuffers& rb) {
  const HfbConfig& cfg = c->cfg;
  int& perSM = c->fineBlocksPerSM[TS == 8 ? 0 : TS == 16 ? 1 : 2][MAXL == 4 ? 0 : MAXL == 8 ? 1 : 2];
  if (perSM == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fineKernel<TS, MAXL>, TS * TS, 0);
  uint32_t grid = cfg.processorCount ? cfg.processorCount : (uint32_t)(max(perSM, 1) * c->smCount);
  uint32_t CAP = cfg.avgFragmentsPerSlice * cfg.slicesPerPixel * cfg.tileSize * cfg.tileSize;
  fineKernel<TS, MAXL><<<grid, TS * TS, 0, c->stream>>>(
      u, h.strandsCount, h.pointsPerStrand, cfg.tileDepthBins, cfg.slicesPerPixel, cfg.shadingPoints, CAP,
      cfg.alphaQuadratic, cfg.alphaMultiplier, (const float4*)pos, (const float4*)tan, (const float4*)shading,
      depth, (const uint4*)rb.tiles, rb.tileSegments, rb.tileList, rb.rasterizerResult,
      (DeviceCounters*)c->dCounters);
  c->launches += 1;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launchTilesPass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                            const float* tan, const float* depth, uint32_t strandsToRender, HfbRasterBuffers& rb) {
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
    tilesRasterKernel<<<divCeil(nSeg, 128), 128, 0, c->stream>>>(
        u, h.pointsPerStrand, nStrands, TS, B, cfg.invalidTilesPerSegmentThreshold, bs, (const float4*)pos,
        (const float4*)tan, depth, (uint4*)rb.tiles, rb.tileSegments, rb.segmentCountPerTile, s.binCount, dc);
  }
  const uint32_t nBlocks = divCeil(TB, SCAN_PER_BLOCK);
  binScanBlocks<<<nBlocks, 512, 0, c->stream>>>(s.binCount, s.binOffset, s.blockSums, TB);
  binScanSums<<<1, 1024, 0, c->stream>>>(s.blockSums, nBlocks);
  binScatterKernel<<<c->smCount * 4, 256, 0, c->stream>>>(rb.tileSegments, rb.maxDrawnSegments, s.binOffset,
                                                          s.blockSums, s.keys, dc);
  binFinalizeKernel<<<min(divCeil(TB, 8), (uint32_t)c->smCount * 16), 256, 0, c->stream>>>(
      TB, s.binCount, s.binOffset, s.blockSums, s.keys, rb.tileSegments, (uint4*)rb.tiles, s.largeBins);
  if (!c->largeBinsAttrSet) {
    e = cudaFuncSetAttribute(largeBinsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, LARGE_SMEM_KEYS * 4);
    if (e != cudaSuccess) return e;
    c->largeBinsAttrSet = true;
  }
  largeBinsKernel<<<c->smCount, 1024, LARGE_SMEM_KEYS * 4, c->stream>>>(
      s.largeBins, s.binCount, s.binOffset, s.blockSums, s.keys, rb.tileSegments, (uint4*)rb.tiles);
  c->launches += nSeg ? 6 : 5;
  return cudaGetLastError();
}

cudaError_t launchTileSort(HfbCtx* c, HfbRasterBuffers& rb) {
  const HfbConfig& cfg = c->cfg;
  const uint32_t T = divCeil(rb.width, cfg.tileSize) * divCeil(rb.height, cfg.tileSize);
  if (cfg.sortBuckets > SORT_MAX_BUCKETS) return cudaErrorInvalidValue;
  tileSortKernel<<<1, 1024, 0, c->stream>>>(T, cfg.sortBuckets, cfg.sortBucketSize, rb.segmentCountPerTile,
                                            rb.sortBuckets, rb.tileList);
  c->launches += 1;
  return cudaGetLastError();
}

cudaError_t launchFinePass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                           const float* tan, const float* shading, const float* depth, HfbRasterBuffers& rb) {
  const uint32_t TS = c->cfg.tileSize, L = c->cfg.slicesPerPixel;
  if (TS == 8) {
    if (L <= 4) return launchFineT<8, 4>(c, u, h, pos, tan, shading, depth, rb);
    if (L <= 8) return launchFineT<8, 8>(c, u, h, pos, tan, shading, depth, rb);
    return launchFineT<8, 16>(c, u, h, pos, tan, shading, depth, rb);
  }
  if (TS == 16) {
    if (L <= 4) return launchFineT<16, 4>(c, u, h, pos, tan, shading, depth, rb);
    if (L <= 8) return launchFineT<16, 8>(c, u, h, pos, tan, shading, depth, rb);
    return launchFineT<16, 16>(c, u, h, pos, tan, shading, depth, rb);
  }
  if (L <= 4) return launchFineT<32, 4>(c, u, h, pos, tan, shading, depth, rb);
  if (L <= 8) return launchFineT<32, 8>(c, u, h, pos, tan, shading, depth, rb);
  return cudaErrorInvalidValue;  // 32x32 tiles with more than 8 slices: too many registers per pixel
}

}  // namespace hfb
