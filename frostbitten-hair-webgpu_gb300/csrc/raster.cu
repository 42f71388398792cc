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

  for (uint32_t ty = tminy; ty <= tmaxy; ty++) {
    for (uint32_t tx = tminx; tx <= tmaxx; tx++) {
      TileB tb = tileBoundsPx(W, H, TS, tx, ty);
      // Only pixel corners inside the segment's bounding rectangle can pass
      // the four edge tests, so the walk is restricted to tile x rect.
      const uint32_t xa = max(tb.x0, ux0), xb = min(tb.x1, ux1 + 1u);
      const uint32_t ya = max(tb.y0, uy0), yb = min(tb.y1, uy1 + 1u);
      float dmin = 999.0f, dmax = -999.0f;
      uint32_t dbin = B;
      for (uint32_t y = ya; y < yb; y++) {
        for (uint32_t x = xa; x < xb; x++) {
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
  if (i == n - 1u) tiles[ti].z = p + 1u;  // head pointer (+1, 0 = empty)
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
constexpr uint32_t CHUNK = 32;

struct FineShared {
  ProjSeg seg[CHUNK];
  uint32_t strand[CHUNK];
  uint32_t segIdx[CHUNK];
  uint32_t cnt[32][CHUNK];  // per-warp passing counts per segment (exact path)
  uint32_t n, nextPtr, queueIdx;
  uint32_t cutSeg, cutSlots, chunkTotal;
};

// Colour of one fragment (processHairSegment.wgsl.ts:43-53), rounded through
// f16 like pack2x16float (hairSlicesDataBuffer.ts:50-63), blended in front of
// the slice's accumulated colour.
template <int MAXL>
__device__ __forceinline__ void addFragment(f4 (&acc)[MAXL], const ProjSeg& s, f2 w, float hd, uint32_t segIdx,
                                            uint32_t strand, uint32_t P, uint32_t SP, uint32_t L, float td0,
                                            float td1, uint32_t alphaQuadratic, float alphaMul,
                                            const float4* __restrict__ shading) {
  // getAlphaCoverage, processHairSegment.wgsl.ts:60-69
  float alpha = fsub(1.0f, fabsf(fsub(fmul(w.x, 2.0f), 1.0f)));
  if (alphaQuadratic) alpha = sqrtf(alpha);
  alpha = sat(fmul(alpha, alphaMul));
  float tFull = fadd((float)segIdx, w.y) / (float)(P - 1u);
  // _sampleShading, hairShadingBuffer.ts:28-38
  uint32_t i0, i1;
  float fr = remapToIndices(SP, tFull, i0, i1);
  const size_t sb = (size_t)strand * SP;
  f4 c = mix4(ld4(__ldg(&shading[sb + i0])), ld4(__ldg(&shading[sb + i1])), fr);
  c.w = fmul(c.w, alpha);
  uint32_t sl = getDepthBin(L, td0, td1, hd);  // getSliceIdx
  f4 q = mk4(__half2float(__float2half_rn(c.x)), __half2float(__float2half_rn(c.y)),
             __half2float(__float2half_rn(c.z)), __half2float(__float2half_rn(c.w)));
  float k = fsub(1.0f, q.w);
#pragma unroll
  for (int si = 0; si < MAXL; si++) {
    if ((uint32_t)si == sl) {
      acc[si].x = fadd(q.x, fmul(k, acc[si].x));
      acc[si].y = fadd(q.y, fmul(k, acc[si].y));
      acc[si].z = fadd(q.z, fmul(k, acc[si].z));
      acc[si].w = fadd(q.w, fmul(k, acc[si].w));
    }
  }
}

// edge + depth test of processHairSegment (:5-31); fills w / hd when it passes
__device__ __forceinline__ bool fragmentPasses(const ProjSeg& s, f2 pp, float zbuf, f2& w, float& hd) {
  if (!insideQuad(s, pp)) return false;
  w = interpolateHairQuad(s, pp);
  hd = interpolateHairF32(w, s.depthsProj);
  return hd < zbuf;  // depth test with GL_LESS (skip when >=)
}

template <int TS, int MAXL>
__global__ void __launch_bounds__(TS * TS)
fineKernel(const HfbUniforms U, uint32_t S, uint32_t P, uint32_t B, uint32_t L, uint32_t SP, uint32_t CAP,
           uint32_t alphaQuadratic, float alphaMul, const float4* __restrict__ pos, const float4* __restrict__ tan,
           const float4* __restrict__ shading, const float* __restrict__ depth, const uint4* __restrict__ tiles,
           const uint32_t* __restrict__ segBuf, const uint32_t* __restrict__ tileList,
           float* __restrict__ result, DeviceCounters* __restrict__ counters) {
  constexpr uint32_t NPX = TS * TS;
  constexpr uint32_t NW = NPX / 32;
  __shared__ FineShared sh;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
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
    __syncthreads();
    if (q >= drawnTiles) break;
    const uint32_t tileIdx = tileList[1u + q];
    if (tileIdx >= tileCount) continue;
    const uint32_t tx = tileIdx % tilesX, ty = tileIdx / tilesX;
    const TileB tbp = tileBoundsPx(W, H, TS, tx, ty);
    const uint32_t px = tbp.x0 + tid % TS, py = tbp.y0 + tid / TS;
    // Pixels of a partial edge tile outside the viewport take no part.
    const bool inView = px < W && py < H;
    const f2 pp = mk2((float)px, (float)py);
    const float zbuf = inView ? loadTex2DClamp(depth, W, H, f2i(pp.x), f2i(fsub(size.y, pp.y))) : 0.0f;
    bool done = !inView;
    f4 fin = mk4(0.f, 0.f, 0.f, 0.f);  // rasterizerResult was cleared before the pass

    for (uint32_t bin = 0; bin < B; bin++) {
      const uint4 head = tiles[ty * tilesX * B + tx * B + bin];
      // _getTileDepth, hairTilesResultBuffer.ts:47-54
      const float td0 = (float)(0xffffffffu - head.x) / F_MAX_U32;
      const float td1 = (float)head.y / F_MAX_U32;
      if (td1 != 0.0f) {  // processTile, :205-288
        f4 acc[MAXL];
#pragma unroll
        for (int si = 0; si < MAXL; si++) acc[si] = mk4(0.f, 0.f, 0.f, 0.f);
        uint32_t nFrag = 0;
        const uint32_t active = __syncthreads_count(!done);
        uint32_t running = 0;  // slots allocated so far (sliceDataOffset)
        uint32_t ptr = head.z == 0u ? INVALID_PTR : head.z - 1u;
        uint32_t processed = 0;
        while (true) {
          // ---- next chunk of the list, read by warp 0 ----
          if (warp == 0) {
            uint32_t p = ptr, n = 0;
            while (n < CHUNK && p != INVALID_PTR && p < maxDrawn && processed + n < maxProcessed) {
              const uint32_t want = min(CHUNK - n, maxProcessed - processed - n);
              // speculate that the list runs p, p-1, p-2, ... (the layout the
              // tiles pass writes); the first entry that does not chain on
              // ends the run and its `next` is followed
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
                sh.strand[n + lane] = e.x & 0x00ffffffu;
                sh.segIdx[n + lane] = e.x >> 24;
              }
              n += cnt;
              p = firstIn ? firstNext : p - cnt;
            }
            if (lane == 0) { sh.n = n; sh.nextPtr = p; }
          }
          __syncthreads();
          const uint32_t n = sh.n;
          if (n == 0) break;
          // ---- project the chunk, one thread per segment ----
          if (tid < n) {
            const uint32_t st = sh.strand[tid], sg = sh.segIdx[tid];
            if (st < S && sg + 1u < P) {
              sh.seg[tid] = projectSegment(U, pos, tan, P, st, sg, size);
            } else {  // not a segment of this hair: covers no pixel
              const float nan = __int_as_float(0x7fffffff);
              sh.seg[tid].v00 = sh.seg[tid].v01 = sh.seg[tid].v10 = sh.seg[tid].v11 = mk2(nan, nan);
              sh.seg[tid].depthsProj = mk4(nan, nan, nan, nan);
            }
          }
          __syncthreads();

          if (running + active * n <= CAP) {
            // ---- fast path: the pool cannot fill inside this chunk ----
            uint32_t myCount = 0;
            if (!done) {
              for (uint32_t j = 0; j < n; j++) {
                f2 w; float hd;
                if (!fragmentPasses(sh.seg[j], pp, zbuf, w, hd)) continue;
                myCount++;
                addFragment<MAXL>(acc, sh.seg[j], w, hd, sh.segIdx[j], sh.strand[j], P, SP, L, td0, td1,
                                  alphaQuadratic, alphaMul, shading);
              }
            }
            nFrag += myCount;
            const uint32_t wsum = __reduce_add_sync(0xffffffffu, myCount);
            if (lane == 0) sh.cnt[warp][0] = wsum;
            __syncthreads();
            uint32_t tot = 0;
#pragma unroll
            for (uint32_t w2 = 0; w2 < NW; w2++) tot += sh.cnt[w2][0];
            running += tot;
          } else {
            // ---- exact path: slots in pixel order, stop at the filling segment ----
            uint32_t mask = 0;
            if (!done) {
              for (uint32_t j = 0; j < n; j++) {
                f2 w; float hd;
                if (fragmentPasses(sh.seg[j], pp, zbuf, w, hd)) mask |= 1u << j;
              }
            }
            for (uint32_t j = 0; j < n; j++) {
              const uint32_t bal = __ballot_sync(0xffffffffu, (mask >> j) & 1u);
              if (lane == 0) sh.cnt[warp][j] = __popc(bal);
            }
            __syncthreads();
            if (warp == 0) {
              uint32_t c = 0;
              if (lane < n)
                for (uint32_t w2 = 0; w2 < NW; w2++) c += sh.cnt[w2][lane];
              uint32_t incl = c;
#pragma unroll
              for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
              }
              const uint32_t fb = __ballot_sync(0xffffffffu, lane < n && running + incl >= CAP);
              const uint32_t j = fb ? (uint32_t)(__ffs(fb) - 1) : 0u;
              const uint32_t exclJ = __shfl_sync(0xffffffffu, incl - c, j);
              const uint32_t total = __shfl_sync(0xffffffffu, incl, n - 1u);
              if (lane == 0) {
                sh.cutSeg = fb ? j : CHUNK;
                sh.cutSlots = fb ? CAP - (running + exclJ) : 0u;
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
              fragmentPasses(sh.seg[j], pp, zbuf, w, hd);
              addFragment<MAXL>(acc, sh.seg[j], w, hd, sh.segIdx[j], sh.strand[j], P, SP, L, td0, td1,
                                alphaQuadratic, alphaMul, shading);
              nFrag++;
            }
            running = cutSeg < CHUNK ? CAP : running + sh.chunkTotal;
          }
          processed += n;
          const uint32_t nextPtr = sh.nextPtr;
          __syncthreads();  // the chunk buffers are refilled next iteration
          if (running >= CAP) {
            if (tid == 0) atomicAdd(&counters->finePoolFullBins, 1ull);
            break;
          }
          ptr = nextPtr;
          if (ptr == INVALID_PTR || ptr >= maxDrawn || processed >= maxProcessed) break;
        }
        // reduceHairSlices (runs for every non-empty bin, as in the reference)
        if (!done) {
          if (isDbg) {
            const uint32_t cntAll = f2u(fmul(fin.x, (float)dbgMax)) + nFrag;
            fin = mk4(sat((float)cntAll / (float)dbgMax), 0.0f, 0.0f, 1.0f);
          } else {
#pragma unroll
            for (int si = 0; si < MAXL; si++) {
              if ((uint32_t)si < L && fin.w < 0.999f) {
                const float k = fsub(1.0f, fin.w);
                fin.x = fadd(fin.x, fmul(acc[si].x, k));
                fin.y = fadd(fin.y, fmul(acc[si].y, k));
                fin.z = fadd(fin.z, fmul(acc[si].z, k));
                fin.w = fadd(fin.w, fmul(acc[si].w, k));
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
  }
}

template <int TS, int MAXL>
cudaError_t launchFineT(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                        const float* tan, const float* shading, const float* depth, HfbRasterBuffers& rb) {
  const HfbConfig& cfg = c->cfg;
  int perSM = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fineKernel<TS, MAXL>, TS * TS, 0);
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
  e = cudaFuncSetAttribute(largeBinsKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, LARGE_SMEM_KEYS * 4);
  if (e != cudaSuccess) return e;
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
