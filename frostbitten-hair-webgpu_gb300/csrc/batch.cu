// Whole frames: one pass of one instance (framePass, the launches of
// hfb_frame), and hfb_frame_batch's batched frame.
//
// A batched frame runs every pass once for all instances: each pass kind
// is one persistent launch over the "virtual blocks" (the blocks the
// single-instance kernel would launch) of every instance.  The host writes
// one prefix row per pass kind over the instances into a device table with
// the instances' pointers and uniforms; everything that changes from one
// batch to the next is data in device memory, so the kernels' launch
// parameters never change and one captured CUDA graph serves every batch of
// the context.
#include <algorithm>
#include <cstring>

#define HFB_TU 5
#include "hfb_internal.cuh"

namespace hfb {

static_assert(BATCH_GROUPS_MAX == sizeof(HfbCtx::batchStreams) / sizeof(cudaStream_t), "group stream table");

// cmdClearBeforeRender of the tiles, fine and sort passes (hairTilesPass.ts:48-52,
// hairFinePass.ts:50-55, hairTileSortPass.ts:63-68).
cudaError_t clearRaster(HfbCtx* c, const HfbRasterBuffers& rb) {
  const HfbConfig& cfg = c->cfg;
  const size_t T = (size_t)divCeil(rb.width, cfg.tileSize) * divCeil(rb.height, cfg.tileSize);
  cudaError_t e = cudaSuccess;
  auto z = [&](void* p, size_t n) { if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, n, c->stream); };
  z(rb.tiles, T * cfg.tileDepthBins * 16);
  z(rb.segmentCountPerTile, T * 4);
  z(rb.tileSegments, 4);
  z(rb.rasterizerResult, 16 + (size_t)rb.width * rb.height * 16);
  z(rb.tileList, 4);
  z(rb.sortBuckets, (size_t)cfg.sortBuckets * 8);
  return e;
}

// One pass of one instance's frame (renderer.ts:171-295).  Integration
// writes positions[1 - current]; every later pass reads those new
// positions, as after HairObject.swapPositionBuffersAfterSimIntegration.
cudaError_t framePass(HfbCtx* c, HfbInstance* in, FramePass p) {
  const HfbSimUniforms& su = *in->simUniforms;
  const HfbUniforms& u = *in->uniforms;
  const HfbHairData& h = in->hair;
  const uint32_t cur = in->current;
  float* prev = in->positions[1u - cur];
  float* now = in->positions[cur];
  HfbRasterBuffers& rb = in->raster;
  switch (p) {
    case FP_GRID_PRE:
      return launchGridPreSim(c, su, in->densityVelocity, in->densityGradWind, in->sdf, in->sdfDims);
    case FP_INTEGRATE:
      if (!h.strandsCount) return cudaSuccess;
      return launchSimIntegrate(c, su, h, prev, now, in->positionsInitial, in->segmentLengths,
                                in->densityVelocity, in->densityGradWind, in->sdf, in->sdfDims);
    case FP_GRID_POST:  // after the swap: "prev" = the old positions, "now" = the new ones
      return launchGridPostSim(c, su, h, now, prev, in->densityVelocity, in->gridOrder);
    case FP_CLEAR:
      return clearRaster(c, rb);
    case FP_TILES: {
      // the segments' projections, for this frame's fine pass
      const cudaError_t e = ensureProjCache(c, (size_t)h.strandsCount * (h.pointsPerStrand - 1u));
      if (e != cudaSuccess) return e;
      return launchTilesPass(c, u, h, prev, in->tangents, in->sceneDepth, in->strandsToRender, rb, c->projCache);
    }
    case FP_SORT:
      return launchTileSort(c, rb);
    case FP_FINE:
      return launchFinePass(c, u, h, prev, in->tangents, in->shading, in->sceneDepth, rb, c->projCache);
    case FP_HAIR_DEPTH:
      if (!in->hairDepth) return cudaSuccess;
      return launchHairDepth(c, u, h, prev, in->tangents, in->strandsToRender, in->sceneDepth, in->hairDepth, rb);
    case FP_SHADING:
      if (!h.strandsCount) return cudaSuccess;
      return launchShading(c, u, h, prev, in->tangents,
                           in->hairDepth ? in->hairDepth : in->shadingDepth ? in->shadingDepth : in->sceneDepth,
                           in->ao, in->ao ? in->aoWidth : 0u, in->ao ? in->aoHeight : 0u, in->shadowMap,
                           in->shadowMap ? in->shadowMapSize : 0u, in->shading);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t ensureProjCache(HfbCtx* c, size_t segments) {
  const size_t need = segments * SEG_PROJ_VEC4 * sizeof(float4);
  if (need <= c->projCacheBytes) return cudaSuccess;
  // the frames in flight may still read the old cache
  cudaError_t e = cudaStreamSynchronize(c->stream);
  for (int i = 0; i < 2 && e == cudaSuccess; i++)
    if (c->pipeStream[i]) e = cudaStreamSynchronize(c->pipeStream[i]);
  for (uint32_t g = 0; g < BATCH_GROUPS_MAX && e == cudaSuccess; g++)
    if (c->batchStreams[g]) e = cudaStreamSynchronize(c->batchStreams[g]);
  if (e != cudaSuccess) return e;
  if (c->projCache) cudaFree(c->projCache);
  c->projCache = nullptr;
  c->projCacheBytes = 0;
  const size_t bytes = need + need / 4;  // room to grow
  e = cudaMalloc(&c->projCache, bytes);
  if (e != cudaSuccess) {
    c->projCache = nullptr;
    return e;
  }
  c->projCacheBytes = bytes;
  return cudaSuccess;
}

namespace {

constexpr uint32_t CLEAR_CHUNK = 65536;  // bytes cleared per virtual block

struct Range {
  unsigned char* p;
  size_t bytes;
};

// What a frame clears for one instance before the raster passes: the
// reference's cmdClearBeforeRender of the tiles, fine and sort passes
// (hairTilesPass.ts:48-52, hairFinePass.ts:50-55, hairTileSortPass.ts:63-68)
// and the tiles pass's own counters.
__host__ __device__ inline uint32_t frameRanges(const HfbConfig& cfg, const BatchInst& I, Range* r) {
  const size_t TB = (size_t)I.T * cfg.tileDepthBins;
  const TilesScratch ts = tilesScratchLayout(I.scratch, cfg, I.W, I.H, I.maxDrawn);
  r[0] = {(unsigned char*)I.tiles, TB * 16};
  r[1] = {(unsigned char*)I.segCount, (size_t)I.T * 4};
  r[2] = {(unsigned char*)I.segBuf, 4};
  r[3] = {(unsigned char*)I.result, 16 + (size_t)I.W * I.H * 16};
  r[4] = {(unsigned char*)I.tileList, 4};
  r[5] = {(unsigned char*)I.sortBuckets, (size_t)cfg.sortBuckets * 8};
  r[6] = {(unsigned char*)ts.binCount, TB * 4};
  r[7] = {(unsigned char*)ts.largeBins, 4};
  return 8;
}

// clearDensityVelocityBuffer of GridPostSimPass (gridPostSimPass.ts:33-59)
__host__ __device__ inline uint32_t gridRanges(const HfbConfig& cfg, const BatchInst& I, Range* r) {
  r[0] = {(unsigned char*)I.dv, (size_t)cfg.gridDims * cfg.gridDims * cfg.gridDims * 16};
  return 1;
}

__host__ __device__ inline uint32_t clearRanges(const HfbConfig& cfg, const BatchInst& I, uint32_t kind,
                                                Range* r) {
  return kind == BK_CLEAR_FRAME ? frameRanges(cfg, I, r) : gridRanges(cfg, I, r);
}

// Zeroes chunk `local` of the instance's ranges: 16-byte stores, then words
// (every range starts 16-byte aligned and is a whole number of words).
__global__ void __launch_bounds__(256) clearBatch(BatchView b, HfbConfig cfgParam, uint32_t kind) {
  const HfbConfig cfg = cfgParam;
  const uint32_t n = b.hdr->n;
  const uint32_t* row = b.prefix + kind * (BATCH_MAX + 1);
  const uint32_t total = row[n];
  for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
    const uint32_t i = batchFind(row, n, v);
    const BatchInst& I = b.insts[i];
    Range r[8];
    const uint32_t nr = clearRanges(cfg, I, kind, r);
    uint32_t c = v - row[i], k = 0;
    for (; k < nr; k++) {
      const uint32_t ch = (uint32_t)((r[k].bytes + CLEAR_CHUNK - 1) / CLEAR_CHUNK);
      if (c < ch) break;
      c -= ch;
    }
    if (k == nr) continue;
    const size_t off = (size_t)c * CLEAR_CHUNK;
    const size_t end = off + CLEAR_CHUNK < r[k].bytes ? off + CLEAR_CHUNK : r[k].bytes;
    unsigned char* p = r[k].p;
    const size_t end16 = off + ((end - off) & ~size_t(15));
    for (size_t x = off + threadIdx.x * 16u; x < end16; x += 256u * 16u)
      *HFB_G(reinterpret_cast<uint4*>(p + x)) = make_uint4(0u, 0u, 0u, 0u);
    for (size_t x = end16 + threadIdx.x * 4u; x < end; x += 256u * 4u) *HFB_G(reinterpret_cast<uint32_t*>(p + x)) = 0u;
  }
}

// sceneDepth -> hairDepth, chunk `local` of the instance's W*H floats; chunk
// 0 also zeroes the count of the hair depth's big-triangle list.
__global__ void __launch_bounds__(256) depthCopyBatch(BatchView b) {
  const uint32_t n = b.hdr->n;
  const uint32_t* row = b.prefix + BK_DEPTH_COPY * (BATCH_MAX + 1);
  const uint32_t total = row[n];
  for (uint32_t v = blockIdx.x; v < total; v += gridDim.x) {
    const uint32_t i = batchFind(row, n, v);
    const BatchInst& I = b.insts[i];
    const size_t bytes = (size_t)I.W * I.H * 4, off = (size_t)(v - row[i]) * CLEAR_CHUNK;
    const size_t end = off + CLEAR_CHUNK < bytes ? off + CLEAR_CHUNK : bytes;
    const unsigned char* src = (const unsigned char*)I.depth;
    unsigned char* dst = (unsigned char*)I.hairDepth;
    for (size_t x = off + threadIdx.x * 4u; x < end; x += 256u * 4u)
      *HFB_G(reinterpret_cast<uint32_t*>(dst + x)) = *HFB_G(reinterpret_cast<const uint32_t*>(src + x));
    if (v == row[i] && threadIdx.x == 0 && I.hdList) *HFB_G(I.hdList) = 0u;
  }
}

}  // namespace

cudaError_t launchBatchDepthCopy(HfbCtx* c, const BatchView& b) {
  HFB_CHECK_BIND(c);
  uint32_t& grid = c->batchGrid[BK_DEPTH_COPY];
  if (!grid) grid = c->smCount * 8u;
  depthCopyBatch<<<batchLaunchGrid(c, grid), 256, 0, c->stream>>>(b);
  HFB_AFTER_LAUNCH(c, "depthCopyBatch");
  c->launches += 1;
  return cudaGetLastError();
}

uint32_t batchBlocks(const HfbConfig& cfg, BatchKind k, const BatchInst& I) {
  const uint32_t G3 = cfg.gridDims * cfg.gridDims * cfg.gridDims;
  const uint32_t TB = I.T * cfg.tileDepthBins;
  const uint32_t nSeg = (I.strandsToRender < I.S ? I.strandsToRender : I.S) * (I.P - 1u);
  switch (k) {
    case BK_CLEAR_FRAME:
    case BK_CLEAR_GRID: {
      Range r[8];
      const uint32_t nr = clearRanges(cfg, I, k, r);
      uint32_t t = 0;
      for (uint32_t j = 0; j < nr; j++) t += (uint32_t)((r[j].bytes + CLEAR_CHUNK - 1) / CLEAR_CHUNK);
      return t;
    }
    case BK_GRID_PRE: return divCeil(G3, 256u);
    case BK_INTEGRATE: return I.S ? divCeil(I.S, simStrandsPerBlock(I.P)) : 0u;
    case BK_GRID_POST: return gridPostBlocks(I.S * I.P);
    case BK_RASTER: return divCeil(nSeg, TILES_RASTER_SEGS);
    case BK_SCAN: return divCeil(TB, 2048u);
    case BK_SCAN_SUMS: return 1u;
    case BK_SCATTER: {
      const uint32_t v = divCeil(nSeg, 1024u);
      return v < 1u ? 1u : (v > 256u ? 256u : v);
    }
    case BK_FINALIZE: return divCeil(TB, 32u);  // a warp takes 4 consecutive bins
    case BK_LARGE: {  // a CTA per bin of more than 1,024 records: more segments, more such bins
      const uint32_t v = divCeil(nSeg, 32768u);
      return v < 4u ? 4u : (v > 64u ? 64u : v);
    }
    case BK_SORT: return 1u;
    case BK_SCHEDULE: return 1u;
    case BK_SHADING: return divCeil(I.S * cfg.shadingPoints, 128u);
    case BK_DEPTH_COPY: return I.hairDepth ? divCeil((uint32_t)(((size_t)I.W * I.H * 4 + CLEAR_CHUNK - 1) / CLEAR_CHUNK), 1u) : 0u;
    case BK_HAIR_DEPTH: return I.hairDepth && I.P > 1u ? hairDepthBlocks(I.S * I.P) : 0u;
    default: return 0u;
  }
}

cudaError_t launchBatchClear(HfbCtx* c, const BatchView& b, BatchKind k) {
  HFB_CHECK_BIND(c);
  uint32_t& grid = c->batchGrid[k];
  if (!grid) grid = c->smCount * 8u;
  clearBatch<<<batchLaunchGrid(c, grid), 256, 0, c->stream>>>(b, c->cfg, (uint32_t)k);
  HFB_AFTER_LAUNCH(c, "clearBatch");
  c->launches += 1;
  return cudaGetLastError();
}

// The frame's launch sequence (renderer.ts:171-295 order): the simulation
// passes, then the raster passes.  With `ev`, an event is recorded before the
// first pass and after each of the HFB_FRAME_PASSES passes (grid_pre,
// integrate, grid_post with its grid clear, clear, tiles, sort, fine,
// hair_depth, shading).
static cudaError_t simSequence(HfbCtx* c, const BatchView& b, cudaEvent_t* ev = nullptr) {
  auto mark = [&](int i) { return ev ? cudaEventRecord(ev[i], c->stream) : cudaSuccess; };
  cudaError_t e = mark(0);
  if (e == cudaSuccess) e = launchBatchSim(c, b, BK_GRID_PRE);
  if (e == cudaSuccess) e = mark(1);
  if (e == cudaSuccess) e = launchBatchSim(c, b, BK_INTEGRATE);
  if (e == cudaSuccess) e = mark(2);
  if (e == cudaSuccess) e = launchBatchClear(c, b, BK_CLEAR_GRID);
  if (e == cudaSuccess) e = launchBatchSim(c, b, BK_GRID_POST);
  if (e == cudaSuccess) e = mark(3);
  return e;
}

static cudaError_t rasterSequence(HfbCtx* c, const BatchView& b, cudaEvent_t* ev = nullptr) {
  auto mark = [&](int i) { return ev ? cudaEventRecord(ev[i], c->stream) : cudaSuccess; };
  cudaError_t e = launchBatchClear(c, b, BK_CLEAR_FRAME);
  if (e == cudaSuccess) e = mark(4);
  if (e == cudaSuccess) e = launchBatchTiles(c, b);
  if (e == cudaSuccess) e = mark(5);
  if (e == cudaSuccess) e = launchBatchSort(c, b);
  if (e == cudaSuccess) e = mark(6);
  if (e == cudaSuccess) e = launchBatchFine(c, b);
  if (e == cudaSuccess) e = mark(7);
  if (e == cudaSuccess) e = launchBatchDepthCopy(c, b);
  if (e == cudaSuccess) e = launchBatchHairDepth(c, b);
  if (e == cudaSuccess) e = mark(8);
  if (e == cudaSuccess) e = launchBatchShading(c, b);
  if (e == cudaSuccess) e = mark(9);
  return e;
}

static cudaError_t batchSequence(HfbCtx* c, const BatchView& b, cudaEvent_t* ev = nullptr) {
  cudaError_t e = simSequence(c, b, ev);
  if (e == cudaSuccess) e = rasterSequence(c, b, ev);
  return e;
}

// One instance as the batched kernels read it.
static void fillInstance(const HfbConfig& cfg, const HfbInstance& s, BatchInst& I) {
  memset(&I, 0, sizeof(I));
  memcpy(&I.U, s.uniforms, sizeof(HfbUniforms));
  memcpy(&I.SU, s.simUniforms, sizeof(HfbSimUniforms));
  I.bsphere = make_float4(s.hair.boundingSphere[0], s.hair.boundingSphere[1], s.hair.boundingSphere[2],
                          s.hair.boundingSphere[3]);
  I.S = s.hair.strandsCount;
  I.P = s.hair.pointsPerStrand;
  I.strandsToRender = s.strandsToRender;
  I.sdfDims = s.sdfDims;
  I.W = s.raster.width;
  I.H = s.raster.height;
  I.maxDrawn = s.raster.maxDrawnSegments;
  I.T = divCeil(I.W, cfg.tileSize) * divCeil(I.H, cfg.tileSize);
  I.aoW = s.ao ? s.aoWidth : 0u;
  I.aoH = s.ao ? s.aoHeight : 0u;
  I.smSize = s.shadowMap ? s.shadowMapSize : 0u;
  I.posNew = (float4*)s.positions[1u - s.current];
  I.posOld = (const float4*)s.positions[s.current];
  I.initial = (const float4*)s.positionsInitial;
  I.tan = (const float4*)s.tangents;
  I.segLen = s.segmentLengths;
  I.dv = (int4*)s.densityVelocity;
  I.gw = (float4*)s.densityGradWind;
  I.sdf = s.sdf;
  I.shading = (float4*)s.shading;
  I.depth = s.sceneDepth;
  I.shadingDepth = s.hairDepth ? s.hairDepth : s.shadingDepth ? s.shadingDepth : s.sceneDepth;
  I.hairDepth = s.hairDepth;
  I.gridOrder = s.gridOrder;
  I.ao = s.ao;
  I.sm = s.shadowMap;
  I.tiles = (uint4*)s.raster.tiles;
  I.segBuf = s.raster.tileSegments;
  I.segCount = s.raster.segmentCountPerTile;
  I.sortBuckets = s.raster.sortBuckets;
  I.tileList = s.raster.tileList;
  I.result = s.raster.rasterizerResult;
  I.scratch = (unsigned char*)s.raster.scratch;
  I.scratchBytes = s.raster.scratchBytes;
  I.hdList = s.hairDepth ? hairDepthList(s.raster.scratch, s.raster.scratchBytes,
                                         rasterPassScratchBytes(cfg, I.W, I.H, s.raster.maxDrawnSegments), &I.hdCap)
                         : nullptr;
  if (!I.hdList) I.hdCap = 0;
}

// Rough GPU work of one instance's frame, for balancing the groups: the
// per-point passes and the per-pixel passes.
static double frameWork(const HfbInstance& in) {
  return (double)in.hair.strandsCount * in.hair.pointsPerStrand +
         0.25 * (double)in.raster.width * in.raster.height;
}

static cudaError_t ensureGroupStreams(HfbCtx* c) {
  cudaError_t e = cudaSuccess;
  if (!c->batchFork) e = cudaEventCreateWithFlags(&c->batchFork, cudaEventDisableTiming);
  for (uint32_t g = 0; g < BATCH_GROUPS_MAX && e == cudaSuccess; g++) {
    if (!c->batchStreams[g]) e = cudaStreamCreateWithFlags(&c->batchStreams[g], cudaStreamNonBlocking);
    if (e == cudaSuccess && !c->batchJoin[g]) e = cudaEventCreateWithFlags(&c->batchJoin[g], cudaEventDisableTiming);
  }
  return e;
}

// The launch sequence of NG groups: one group on c->stream, or each group
// on its own worker stream, forked from c->stream and joined back into it.
static cudaError_t groupsSequence(HfbCtx* c, uint32_t NG) {
  if (NG == 1) return batchSequence(c, batchView(c->batchDev));
  const cudaStream_t caller = c->stream;
  cudaError_t e = cudaEventRecord(c->batchFork, caller);
  for (uint32_t g = 0; g < NG && e == cudaSuccess; g++) e = cudaStreamWaitEvent(c->batchStreams[g], c->batchFork, 0);
  if (e != cudaSuccess) return e;
  c->batchGridDiv = NG;
  for (uint32_t g = 0; g < NG && e == cudaSuccess; g++) {
    c->stream = c->batchStreams[g];
    e = batchSequence(c, batchView((char*)c->batchDev + (size_t)g * BATCH_BYTES));
  }
  c->stream = caller;
  c->batchGridDiv = 1;
  for (uint32_t g = 0; g < NG; g++) {  // also after a failed launch: the streams stay joined
    cudaError_t ej = cudaEventRecord(c->batchJoin[g], c->batchStreams[g]);
    if (ej == cudaSuccess) ej = cudaStreamWaitEvent(caller, c->batchJoin[g], 0);
    if (e == cudaSuccess) e = ej;
  }
  return e;
}

// Pipelined batches: the device table slots after the groups' tables.
static char* pipeTable(HfbCtx* c, uint32_t slot) {
  return (char*)c->batchDev + (size_t)(BATCH_GROUPS_MAX + slot) * BATCH_BYTES;
}

static cudaError_t ensurePipe(HfbCtx* c) {
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 && e == cudaSuccess; i++) {
    if (!c->pipeStream[i]) e = cudaStreamCreateWithFlags(&c->pipeStream[i], cudaStreamNonBlocking);
    if (e == cudaSuccess && !c->pipeSimDone[i]) e = cudaEventCreateWithFlags(&c->pipeSimDone[i], cudaEventDisableTiming);
    if (e == cudaSuccess && !c->pipeRasterDone[i])
      e = cudaEventCreateWithFlags(&c->pipeRasterDone[i], cudaEventDisableTiming);
    if (e == cudaSuccess && !c->pipeCaller[i]) e = cudaEventCreateWithFlags(&c->pipeCaller[i], cudaEventDisableTiming);
  }
  return e;
}

static void pipeGraphsRelease(HfbCtx* c) {
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      if (c->pipeGraph[i][j]) cudaGraphExecDestroy(c->pipeGraph[i][j]);
      c->pipeGraph[i][j] = nullptr;
    }
}

// One half of a pipelined frame (part 0: simulation, 1: raster) on its
// stream: plain launches for the first use of each table slot (they also set
// the kernels' attributes), then the slot's captured graph.
static cudaError_t pipePart(HfbCtx* c, uint32_t part, uint32_t slot) {
  const cudaStream_t caller = c->stream;
  c->stream = c->pipeStream[part];
  const BatchView b = batchView(pipeTable(c, slot));
  auto seq = [&]() { return part == 0u ? simSequence(c, b) : rasterSequence(c, b); };
  cudaError_t e = cudaSuccess;
#ifdef HFB_DEVICE_CHECKS
  const bool plain = true;  // the checked build waits after every launch: no capture
#else
  const bool plain = c->pipeCalls <= 2u;
#endif
  if (plain) {
    e = seq();
  } else {
    cudaGraphExec_t& ge = c->pipeGraph[slot][part];
    if (!ge) {
      cudaGraph_t gr = nullptr;
      e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        const uint64_t l0 = c->launches;
        cudaError_t el = seq();
        c->pipeGraphLaunches[slot][part] = c->launches - l0;
        c->launches = l0;
        e = cudaStreamEndCapture(c->stream, &gr);
        if (el != cudaSuccess) e = el;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, gr, 0);
        if (gr) cudaGraphDestroy(gr);
      }
    }
    if (e == cudaSuccess) {
      e = cudaGraphLaunch(ge, c->stream);
      c->launches += c->pipeGraphLaunches[slot][part];
    }
  }
  c->stream = caller;
  return e;
}

// Fills the staging copy (one device table per group), uploads it and runs
// the frame for n validated instances.
cudaError_t frameBatch(HfbCtx* c, HfbInstance* insts, uint32_t n, float* passMs) {
  cudaError_t e = cudaSuccess;
  constexpr size_t TABLES = (size_t)(BATCH_GROUPS_MAX + 2) * BATCH_BYTES;  // groups + two pipeline slots
  if (!c->batchDev) {
    e = cudaMalloc(&c->batchDev, TABLES);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
      e = cudaMallocHost(&c->batchHost[k], TABLES);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->batchCopied[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(c->batchCopied[k], c->stream);
    }
    if (e == cudaSuccess) e = ensureGroupStreams(c);
    if (e != cudaSuccess) return e;
  }
  // groups: largest instance first, each to the group with the least work so
  // far (the profiling run keeps one group: its passes are timed one by one)
  const bool pipe = c->batchPipeline && !passMs;
  uint32_t NG = (passMs || pipe) ? 1u : (c->batchGroups < n ? c->batchGroups : n);
  if (NG < 1u) NG = 1u;
  uint32_t* group = new uint32_t[n];
  {
    uint32_t* order = new uint32_t[n];
    for (uint32_t i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order, order + n, [&](uint32_t a, uint32_t b) { return frameWork(insts[a]) > frameWork(insts[b]); });
    double load[BATCH_GROUPS_MAX] = {};
    for (uint32_t k = 0; k < n; k++) {
      const uint32_t i = order[k];
      const uint32_t g = (uint32_t)(std::min_element(load, load + NG) - load);
      load[g] += frameWork(insts[i]);
      group[i] = g;
    }
    delete[] order;
  }
  // the staging copy is rewritten once its previous upload has been read
  const uint32_t k = c->batchFlip;
  c->batchFlip ^= 1u;
  e = cudaEventSynchronize(c->batchCopied[k]);
  if (e != cudaSuccess) { delete[] group; return e; }
  const HfbConfig& cfg = c->cfg;
  // the frame's projected segments: one region per instance, written by the
  // tiles pass and read by the fine pass
  size_t segs = 0;
  for (uint32_t i = 0; i < n; i++) segs += (size_t)insts[i].hair.strandsCount * (insts[i].hair.pointsPerStrand - 1u);
  e = ensureProjCache(c, segs);
  if (e != cudaSuccess) { delete[] group; return e; }
  uint32_t ng[BATCH_GROUPS_MAX] = {};
  size_t smem = c->simBatchSmem, segOff = 0;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t g = group[i];
    char* h = (char*)c->batchHost[k] + (size_t)g * BATCH_BYTES;
    BatchInst& I = ((BatchInst*)(h + BATCH_INSTS_OFF))[ng[g]++];
    fillInstance(cfg, insts[i], I);
    I.proj = c->projCache + segOff * SEG_PROJ_VEC4;
    segOff += (size_t)insts[i].hair.strandsCount * (insts[i].hair.pointsPerStrand - 1u);
    const size_t sb = simSmemBytes(insts[i].hair.pointsPerStrand);
    smem = smem > sb ? smem : sb;
  }
  delete[] group;
  // the integration launch stages the longest strands of the batch: a batch
  // with longer strands than any before it re-sizes it (and the graph)
  if (smem > c->simBatchSmem) {
    c->simBatchSmem = smem;
    c->batchGrid[BK_INTEGRATE] = 0;
    e = cudaStreamSynchronize(c->stream);
    for (int i = 0; i < 2 && e == cudaSuccess; i++)
      if (c->pipeStream[i]) e = cudaStreamSynchronize(c->pipeStream[i]);
    if (e != cudaSuccess) return e;
    if (c->batchGraph) cudaGraphExecDestroy(c->batchGraph);
    c->batchGraph = nullptr;
    pipeGraphsRelease(c);
  }
  for (uint32_t g = 0; g < NG && e == cudaSuccess; g++) {
    char* h = (char*)c->batchHost[k] + (size_t)g * BATCH_BYTES;
    BatchHdr* hdr = (BatchHdr*)h;
    memset(hdr, 0, sizeof(*hdr));
    hdr->n = ng[g];
    uint32_t* prefix = (uint32_t*)(h + BATCH_PREFIX_OFF);
    const BatchInst* bi = (const BatchInst*)(h + BATCH_INSTS_OFF);
    for (uint32_t kind = 0; kind < BK_COUNT; kind++) {
      uint32_t* row = prefix + (size_t)kind * (BATCH_MAX + 1);
      uint32_t acc = 0;
      for (uint32_t i = 0; i < ng[g]; i++) {
        row[i] = acc;
        acc += batchBlocks(cfg, (BatchKind)kind, bi[i]);
      }
      row[ng[g]] = acc;
    }
    if (pipe) break;  // uploaded on the simulation stream below
    const size_t bytes = BATCH_INSTS_OFF + (size_t)ng[g] * sizeof(BatchInst);
    e = cudaMemcpyAsync((char*)c->batchDev + (size_t)g * BATCH_BYTES, h, bytes, cudaMemcpyHostToDevice, c->stream);
  }
  if (e != cudaSuccess) return e;
  if (pipe) {
    // Table slot k.  The frame's simulation waits for the caller's stream as
    // of the previous call (or this one, the first time) and for the raster
    // passes of the frame before the previous one, which read the table slot
    // and the position buffer this simulation writes; it runs beside the
    // previous frame's raster passes.  The raster passes wait for this
    // simulation and, on their own stream, for the previous raster passes;
    // the caller's stream waits for them.
    e = ensurePipe(c);
    if (e == cudaSuccess) e = cudaEventRecord(c->pipeCaller[k], c->stream);
    const cudaStream_t S = c->pipeStream[0], R = c->pipeStream[1];
    if (e == cudaSuccess) e = cudaStreamWaitEvent(S, c->pipeCaller[c->pipeCalls == 0 ? k : 1u - k], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(S, c->pipeRasterDone[k], 0);
    const size_t bytes = BATCH_INSTS_OFF + (size_t)n * sizeof(BatchInst);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pipeTable(c, k), c->batchHost[k], bytes, cudaMemcpyHostToDevice, S);
    if (e == cudaSuccess) e = cudaEventRecord(c->batchCopied[k], S);
    c->pipeCalls++;
    if (e == cudaSuccess) e = pipePart(c, 0, k);
    if (e == cudaSuccess) e = cudaEventRecord(c->pipeSimDone[k], S);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(R, c->pipeSimDone[k], 0);
    if (e == cudaSuccess) e = pipePart(c, 1, k);
    if (e == cudaSuccess) e = cudaEventRecord(c->pipeRasterDone[k], R);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->pipeRasterDone[k], 0);
    if (e != cudaSuccess) return e;
    for (uint32_t i = 0; i < n; i++) insts[i].current ^= 1u;
    return cudaGetLastError();
  }
  e = cudaEventRecord(c->batchCopied[k], c->stream);
  if (e != cudaSuccess) return e;

  if (passMs) {  // one group, plain launches with an event between passes
    cudaEvent_t ev[HFB_FRAME_PASSES + 1] = {};
    for (int i = 0; i <= HFB_FRAME_PASSES && e == cudaSuccess; i++) e = cudaEventCreate(&ev[i]);
    if (e == cudaSuccess) e = batchSequence(c, batchView(c->batchDev), ev);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[HFB_FRAME_PASSES]);
    for (int i = 0; i < HFB_FRAME_PASSES && e == cudaSuccess; i++) e = cudaEventElapsedTime(&passMs[i], ev[i], ev[i + 1]);
    for (int i = 0; i <= HFB_FRAME_PASSES; i++)
      if (ev[i]) cudaEventDestroy(ev[i]);
    if (e != cudaSuccess) return e;
    for (uint32_t i = 0; i < n; i++) insts[i].current ^= 1u;
    return cudaGetLastError();
  }
#ifdef HFB_DEVICE_CHECKS
  c->batchGraphLaunches = ~0ull;  // the checked build waits after every launch: no capture
#endif
  if (c->batchGraph && c->batchGraphGroups != NG) {  // made for another number of groups
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return e;
    cudaGraphExecDestroy(c->batchGraph);
    c->batchGraph = nullptr;
  }
  if (c->batchCalls++ == 0 || c->batchGraphLaunches == ~0ull) {
    // the first batch (which also sets the kernels' attributes), or no graph: plain launches
    e = groupsSequence(c, NG);
  } else {
    if (!c->batchGraph) {
      cudaGraph_t gr = nullptr;
      e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return e;
      const uint64_t l0 = c->launches;
      cudaError_t el = groupsSequence(c, NG);
      const uint64_t captured = c->launches - l0;
      c->launches = l0;
      e = cudaStreamEndCapture(c->stream, &gr);
      if (el != cudaSuccess) e = el;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&c->batchGraph, gr, 0);
      if (gr) cudaGraphDestroy(gr);
      if (e != cudaSuccess) {
        // a stream that cannot be captured (e.g. the legacy default stream): plain launches
        cudaGetLastError();
        c->batchGraph = nullptr;
        c->batchGraphLaunches = ~0ull;
        e = groupsSequence(c, NG);
        if (e != cudaSuccess) return e;
        for (uint32_t i = 0; i < n; i++) insts[i].current ^= 1u;
        return cudaGetLastError();
      }
      c->batchGraphLaunches = captured;
      c->batchGraphGroups = NG;
    }
    e = cudaGraphLaunch(c->batchGraph, c->stream);
    c->launches += c->batchGraphLaunches;
  }
  if (e != cudaSuccess) return e;
  for (uint32_t i = 0; i < n; i++) insts[i].current ^= 1u;
  return cudaGetLastError();
}

void frameBatchRelease(HfbCtx* c) {
  pipeGraphsRelease(c);
  for (int i = 0; i < 2; i++) {
    if (c->pipeStream[i]) cudaStreamDestroy(c->pipeStream[i]);
    for (cudaEvent_t* ev : {&c->pipeSimDone[i], &c->pipeRasterDone[i], &c->pipeCaller[i]}) {
      if (*ev) cudaEventDestroy(*ev);
      *ev = nullptr;
    }
    c->pipeStream[i] = nullptr;
  }
  for (uint32_t g = 0; g < BATCH_GROUPS_MAX; g++) {
    if (c->batchJoin[g]) cudaEventDestroy(c->batchJoin[g]);
    if (c->batchStreams[g]) cudaStreamDestroy(c->batchStreams[g]);
    c->batchJoin[g] = nullptr;
    c->batchStreams[g] = nullptr;
  }
  if (c->batchFork) cudaEventDestroy(c->batchFork);
  c->batchFork = nullptr;
  if (c->batchGraph) cudaGraphExecDestroy(c->batchGraph);
  for (int k = 0; k < 2; k++) {
    if (c->batchCopied[k]) cudaEventDestroy(c->batchCopied[k]);
    if (c->batchHost[k]) cudaFreeHost(c->batchHost[k]);
  }
  if (c->batchDev) cudaFree(c->batchDev);
  c->batchGraph = nullptr;
  c->batchDev = nullptr;
  if (c->projCache) cudaFree(c->projCache);
  c->projCache = nullptr;
  c->projCacheBytes = 0;
}

}  // namespace hfb
