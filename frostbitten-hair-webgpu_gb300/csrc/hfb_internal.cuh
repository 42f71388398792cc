// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/hairfb.h"

#include "hfb_check.cuh"

struct HfbCtx {
  HfbConfig cfg;
  int device = 0;
  int smCount = 0;
  cudaStream_t ownStream = nullptr;
  cudaStream_t stream = nullptr;
  std::string lastError;
  // device-side counters: HfbDeviceCounters
  unsigned long long* dCounters = nullptr;
  uint64_t launches = 0;
  // per-context launch set-up done once (kernel attributes, occupancy)
  bool largeBinsAttrSet = false;
  int fineBlocksPerSM[3][3] = {};  // [tile 8/16/32][slices 4/8/16]
  // batched frames: device table + two pinned host staging copies, the
  // persistent grid of each batched kernel, the captured frame graph
  void* batchDev = nullptr;
  void* batchHost[2] = {nullptr, nullptr};
  cudaEvent_t batchCopied[2] = {nullptr, nullptr};
  uint32_t batchFlip = 0;
  uint32_t batchGrid[32] = {};
  cudaGraphExec_t batchGraph = nullptr;
  uint64_t batchGraphLaunches = 0;  // kernels in the graph
  uint32_t batchCalls = 0;
  size_t simBatchSmem = 0;  // shared memory of the batched integration launch
  // groups of a batched frame: each group's passes on its own worker stream,
  // its persistent launches sized to 1 / groups of the GPU
  uint32_t batchGroups = 1;       // requested (hfb_ctx_set_batch_groups)
  uint32_t batchGraphGroups = 0;  // groups the captured graph was made with
  uint32_t batchGridDiv = 1;      // divisor of the persistent grids while a group launches
  cudaStream_t batchStreams[4] = {};
  cudaEvent_t batchFork = nullptr;
  cudaEvent_t batchJoin[4] = {};
  // pipelined batches (hfb_ctx_set_batch_pipeline): the simulation passes on
  // one stream, the raster passes on another, two device tables in turn
  bool batchPipeline = false;
  uint64_t pipeCalls = 0;
  cudaStream_t pipeStream[2] = {};         // [0] simulation, [1] raster
  cudaEvent_t pipeSimDone[2] = {};         // per table slot
  cudaEvent_t pipeRasterDone[2] = {};
  cudaEvent_t pipeCaller[2] = {};          // the caller's stream at each call
  cudaGraphExec_t pipeGraph[2][2] = {};    // [slot][simulation / raster]
  uint64_t pipeGraphLaunches[2][2] = {};
  // self-checking build: the device CheckState (hfb_check.cuh), else NULL
  void* checkDev = nullptr;
  // device address of hfb_tiles_pass_noalloc's fixed array on this
  // context's device, looked up when the context is created (NULL if that
  // failed; noallocError then says why)
  void* noallocScratch = nullptr;
  std::string noallocError;
  // the projected segments of a whole frame (hfb_frame, hfb_frame_batch):
  // written by the tiles pass, read by the fine pass; grown on demand
  float4* projCache = nullptr;
  size_t projCacheBytes = 0;
};

namespace hfb {

// Device counters, mirrored into HfbCounters by hfb_get_counters.
struct DeviceCounters {
  unsigned long long tileRecords;
  unsigned long long tileRecordsDropped;
  unsigned long long finePoolFullBins;
  unsigned long long fineSplitTiles;
  unsigned long long fineSplitRedone;
  unsigned long long badWorkItems;
};

// Layout of the tiles-pass scratch area (all offsets 256-byte aligned).
struct TilesScratch {
  uint32_t* binCount;    // T*B counts of records per (tile, depth bin)
  uint32_t* binOffset;   // T*B exclusive prefix of binCount, then cursor
  uint32_t* keys;        // maxDrawn sort keys (strand << 8 | segment), CSR order
  uint32_t* blockSums;   // scan partials
  uint32_t* largeBins;   // [0] = count, then bin indices with > 1024 records
  size_t bytes;
};

// Layout of the fine-pass scratch area (the same memory as the tiles pass's,
// which is dead by then; all offsets 256-byte aligned).
struct FineScratch {
  uint32_t* hdr;       // [0] = work items
  uint4* items;        // tile list index, b0 | b1 << 8 | group << 16 | groups << 24, first group slot
  uint32_t* arrivals;  // per split tile (at its first group slot): groups done | 1 << 31 if one gave up
  float4* groups;      // per group slot: the TS*TS composites of the group's depth bins
  uint32_t maxItems, maxGroups;
  size_t bytes;
};
uint32_t maxDrawnSegments(const HfbConfig& cfg, uint32_t W, uint32_t H);

// Strands per integration block for P points per strand: 2048 / P, between
// 8 and 128, so a block's 128 threads take sixteen points each in the point
// phases and its staging (the points only) stays near 34 KB: 64 strands of
// 32 points, 128 of 16.
__host__ __device__ inline uint32_t simStrandsPerBlock(uint32_t P) {
  const uint32_t n = 2048u / P;
  return n > 128u ? 128u : n < 8u ? 8u : n;
}
// The same for one instance launched alone (hfb_sim_integrate, hfb_frame):
// fewer strands per block (at least 8) while that gives up to two blocks per SM.
__host__ __device__ inline uint32_t simStrandsPerBlockFor(uint32_t S, uint32_t P, uint32_t smCount) {
  const uint32_t full = simStrandsPerBlock(P);
  const uint32_t want = (S + 2u * smCount - 1u) / (2u * smCount);  // strands per block for 2 blocks per SM
  return want >= full ? full : want < 8u ? 8u : want;
}
__host__ __device__ inline size_t simSmemBytes(uint32_t P) {
  return (size_t)simStrandsPerBlock(P) * (P + 1u) * sizeof(float4) + (size_t)P * 4u;
}
constexpr uint32_t TILES_RASTER_SEGS = 128;  // segments per tiles-raster block

// Launchers. Each returns cudaSuccess or the launch error.
cudaError_t launchGridPreSim(HfbCtx* c, const HfbSimUniforms& u, const int32_t* dv, float* gw,
                             const float* sdf, uint32_t sdfDims);
cudaError_t launchSimIntegrate(HfbCtx* c, const HfbSimUniforms& u, const HfbHairData& h, float* prev,
                               const float* now, const float* initial, const float* segLen,
                               const int32_t* dv, const float* gw, const float* sdf, uint32_t sdfDims);
cudaError_t launchGridPostSim(HfbCtx* c, const HfbSimUniforms& u, const HfbHairData& h, const float* prev,
                              const float* now, int32_t* dv, const uint32_t* strandOrder);
cudaError_t launchShading(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                          const float* tan, const float* depth, const float* ao, uint32_t aoW,
                          uint32_t aoH, const float* sm, uint32_t smSize, float* shading);
// proj (NULL = none): per segment, SEG_PROJ_VEC4 float4 of its projection
// (projectSegment) that the tiles pass writes and the fine pass of the same
// frame reads instead of projecting again (whole frames only, where the
// library runs both passes on the same positions and uniforms).
constexpr uint32_t SEG_PROJ_VEC4 = 3;  // v00, v01 | v10, v11 | depthsProj
cudaError_t launchTilesPass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                            const float* tan, const float* depth, uint32_t strandsToRender,
                            HfbRasterBuffers& rb, float4* proj = nullptr);
cudaError_t launchTileSort(HfbCtx* c, HfbRasterBuffers& rb);
cudaError_t launchFinePass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                           const float* tan, const float* shading, const float* depth,
                           HfbRasterBuffers& rb, const float4* proj = nullptr);

__host__ __device__ inline uint32_t divCeil(uint32_t a, uint32_t b) { return (a + b - 1u) / b; }
__host__ __device__ inline size_t alignUp256(size_t v) { return (v + 255u) & ~size_t(255u); }

__host__ __device__ inline TilesScratch tilesScratchLayout(void* base, const HfbConfig& cfg, uint32_t W,
                                                           uint32_t H, uint32_t maxDrawn) {
  const size_t T = (size_t)divCeil(W, cfg.tileSize) * divCeil(H, cfg.tileSize);
  const size_t TB = T * cfg.tileDepthBins;
  const size_t nBlocks = (TB + 2047) / 2048 + 1;
  char* p = (char*)base;
  TilesScratch s;
  size_t off = 0;
  s.binCount = (uint32_t*)(p + off); off = alignUp256(off + TB * 4);
  s.binOffset = (uint32_t*)(p + off); off = alignUp256(off + TB * 4);
  s.keys = (uint32_t*)(p + off); off = alignUp256(off + (size_t)maxDrawn * 4);
  s.blockSums = (uint32_t*)(p + off); off = alignUp256(off + nBlocks * 4 + 16);
  s.largeBins = (uint32_t*)(p + off); off = alignUp256(off + (TB + 1) * 4);
  s.bytes = off;
  return s;
}

__host__ __device__ inline FineScratch fineScratchLayout(void* base, const HfbConfig& cfg, uint32_t W,
                                                         uint32_t H) {
  const size_t T = (size_t)divCeil(W, cfg.tileSize) * divCeil(H, cfg.tileSize);
  const size_t groupBytes = (size_t)cfg.tileSize * cfg.tileSize * 16;
  FineScratch s;
  // split groups: at most 1024, and at most 4 MiB of composites
  const size_t byBytes = ((size_t)4 << 20) / groupBytes;
  s.maxGroups = (uint32_t)(byBytes < 1024 ? byBytes : 1024);
  s.maxItems = (uint32_t)(T + s.maxGroups);
  char* p = (char*)base;
  size_t off = 0;
  s.hdr = (uint32_t*)(p + off); off = alignUp256(off + 16);
  s.items = (uint4*)(p + off); off = alignUp256(off + (size_t)s.maxItems * 16);
  s.arrivals = (uint32_t*)(p + off); off = alignUp256(off + (size_t)s.maxGroups * 4);
  s.groups = (float4*)(p + off); off = alignUp256(off + (size_t)s.maxGroups * groupBytes);
  s.bytes = off;
  return s;
}

// ---------------------------------------------------------------------------
// Whole frames.  A frame of one instance (hfb_frame) is the reference's pass
// sequence; framePass launches one pass of it on c->stream.
// ---------------------------------------------------------------------------
enum FramePass : uint32_t {
  FP_GRID_PRE = 0,  // GridPreSimPass
  FP_INTEGRATE,     // HairSimIntegrationPass
  FP_GRID_POST,     // GridPostSimPass (with its grid clear)
  FP_CLEAR,         // cmdClearBeforeRender of the raster passes
  FP_TILES,         // HairTilesPass
  FP_SORT,          // HairTileSortPass
  FP_FINE,          // HairFinePass
  FP_HAIR_DEPTH,    // HwHairPass's depth (only for instances with hairDepth)
  FP_SHADING,       // HairShadingPass
  FP_COUNT
};
cudaError_t framePass(HfbCtx* c, HfbInstance* in, FramePass p);
cudaError_t clearRaster(HfbCtx* c, const HfbRasterBuffers& rb);

// Looks up the device address of hfb_tiles_pass_noalloc's fixed array with
// the context's device current (noalloc.cu), which also loads that code
// onto the device and makes the array resident; called by hfb_ctx_create.
// Sets c->noallocScratch, or c->noallocError on failure.
void noallocPrepare(HfbCtx* c);
// Makes c->projCache hold at least `segments` projected segments (waits for
// the context's streams before replacing a smaller one).
cudaError_t ensureProjCache(HfbCtx* c, size_t segments);
// Loads the tiles pass's kernels onto the current device (raster.cu).
cudaError_t tilesPassLoad(HfbCtx* c);

// ---------------------------------------------------------------------------
// Batched frames (hfb_frame_batch): every pass runs once for all instances.
// Each batched kernel is persistent and walks "virtual blocks": instance i
// owns virtual blocks [prefix[k][i], prefix[k][i + 1]) of kind k, and block
// v of instance i runs the single-instance kernel's body as its block
// v - prefix[k][i].  Instances, prefix rows and counters live in device
// memory, so the launch sequence is the same for every batch and is
// captured once as a CUDA graph.
// ---------------------------------------------------------------------------
constexpr uint32_t BATCH_MAX = 1024;  // instances per batch
constexpr uint32_t BATCH_GROUPS_MAX = 4;
// Grid of one persistent batched launch: the full-GPU grid `full`, divided
// among the groups that run side by side.
inline uint32_t batchLaunchGrid(const HfbCtx* c, uint32_t full) {
  const uint32_t g = full / c->batchGridDiv;
  return g ? g : 1u;
}
enum BatchKind : uint32_t {
  BK_CLEAR_FRAME = 0,  // raster clears + tiles-pass counters
  BK_GRID_PRE,
  BK_INTEGRATE,
  BK_CLEAR_GRID,       // densityVelocity, after integration read it
  BK_GRID_POST,
  BK_RASTER,
  BK_SCAN,
  BK_SCAN_SUMS,
  BK_SCATTER,
  BK_FINALIZE,
  BK_LARGE,
  BK_SORT,
  BK_SCHEDULE,
  BK_SHADING,
  BK_DEPTH_COPY,       // sceneDepth -> hairDepth (and the big-triangle list's count)
  BK_HAIR_DEPTH,
  BK_COUNT
};

// One instance of a batched frame, as the kernels read it.
struct alignas(16) BatchInst {
  HfbUniforms U;
  HfbSimUniforms SU;
  float4 bsphere;
  uint32_t S, P, strandsToRender, sdfDims;
  uint32_t W, H, maxDrawn, T;
  uint32_t aoW, aoH, smSize, pad0;
  float4* posNew;        // positions[1 - current]: integration writes it, the raster reads it
  const float4* posOld;  // positions[current]
  const float4* initial;
  const float4* tan;
  const float* segLen;
  int4* dv;
  float4* gw;
  const float* sdf;
  float4* shading;
  const float* depth;         // scene depth of the tiles / fine depth tests
  const float* shadingDepth;  // depth of the shading attenuation
  const float* ao;
  const float* sm;
  uint4* tiles;
  uint32_t* segBuf;
  uint32_t* segCount;
  uint32_t* sortBuckets;
  uint32_t* tileList;
  float* result;
  unsigned char* scratch;
  size_t scratchBytes;
  float* hairDepth;           // NULL: no hair depth prepass
  uint32_t* hdList;           // the hair depth pass's big-triangle list (word 0: count), or NULL
  uint32_t hdCap, pad1;
  const uint32_t* gridOrder;  // strand order of the grid splat, NULL = identity
  float4* proj;               // the frame's projected segments (SEG_PROJ_VEC4 each), or NULL
};

// Device layout of a batch: header, prefix rows (fixed stride), the fine
// pass's item prefix, the instances.
struct BatchHdr {
  uint32_t n;
  uint32_t fineQueue;  // next global work item of the batched fine pass
  uint32_t pad[2];
  uint32_t queue[BK_COUNT];  // next virtual block of each kind (batchNext)
};
static_assert(sizeof(BatchHdr) <= 256, "the batch header fits before the prefix rows");
constexpr size_t BATCH_PREFIX_OFF = 256;
constexpr size_t BATCH_ITEMS_OFF = BATCH_PREFIX_OFF + (size_t)BK_COUNT * (BATCH_MAX + 1) * 4;
constexpr size_t BATCH_INSTS_OFF = (BATCH_ITEMS_OFF + (size_t)(BATCH_MAX + 1) * 4 + 255) & ~size_t(255);
constexpr size_t BATCH_BYTES = BATCH_INSTS_OFF + (size_t)BATCH_MAX * sizeof(BatchInst);

struct BatchView {
  BatchHdr* hdr;
  const uint32_t* prefix;  // [BK_COUNT][BATCH_MAX + 1]
  uint32_t* itemPrefix;    // [BATCH_MAX + 1]
  const BatchInst* insts;
};
inline BatchView batchView(void* base) {
  char* p = (char*)base;
  return {(BatchHdr*)p, (const uint32_t*)(p + BATCH_PREFIX_OFF), (uint32_t*)(p + BATCH_ITEMS_OFF),
          (const BatchInst*)(p + BATCH_INSTS_OFF)};
}

// Instance owning virtual block v: the last i with row[i] <= v (row[n] = total).
__device__ __forceinline__ uint32_t batchFind(const uint32_t* __restrict__ row, uint32_t n, uint32_t v) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1u) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&row[mid]) <= v) lo = mid; else hi = mid;
  }
  return lo;
}

// The next virtual block of kind k for the calling CTA, from the header's
// counter (zeroed by every frame's table upload): CTAs take blocks as they
// finish, so uneven blocks do not leave some CTAs with a long tail.  Every
// thread of the CTA calls it; `slots` are two shared words used in turn
// (`parity`, per thread): the write of a call can only meet reads of the
// call two before, which every thread finished before the barrier of the
// call in between.  The barrier also orders a block body's shared-memory
// reads before the next body's writes.
__device__ __forceinline__ uint32_t batchNext(BatchHdr* hdr, uint32_t k, uint32_t* slots, uint32_t& parity) {
  if (threadIdx.x == 0) slots[parity] = atomicAdd(&hdr->queue[k], 1u);
  __syncthreads();
  const uint32_t v = slots[parity];
  parity ^= 1u;
  return v;
}

// Batched launchers: one persistent launch of kind k over all instances.
cudaError_t launchBatchClear(HfbCtx* c, const BatchView& b, BatchKind k);
cudaError_t launchBatchSim(HfbCtx* c, const BatchView& b, BatchKind k);
// hfb_check_constant_division: cnt[3] on the device, zeroed here
cudaError_t launchConstDivCheck(HfbCtx* c, unsigned long long* cnt);
cudaError_t launchBatchShading(HfbCtx* c, const BatchView& b);
cudaError_t launchBatchTiles(HfbCtx* c, const BatchView& b);
cudaError_t launchBatchSort(HfbCtx* c, const BatchView& b);
cudaError_t launchBatchFine(HfbCtx* c, const BatchView& b);
cudaError_t launchBatchHairDepth(HfbCtx* c, const BatchView& b);
cudaError_t launchBatchDepthCopy(HfbCtx* c, const BatchView& b);
// Hair depth prepass (hairdepth.cu); entries of its big-triangle list in a
// raster scratch area of `bytes` (word 0 = count).
cudaError_t launchHairDepth(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos, const float* tan,
                            uint32_t strandsToRender, const float* sceneDepth, float* hairDepth,
                            HfbRasterBuffers& rb);
cudaError_t launchHairNormals(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos, const float* tan,
                              uint32_t strandsToRender, const float* hairDepth, float* normals, uint32_t* winner,
                              HfbRasterBuffers& rb);
// AO texture extent: ceil(viewport * scale), as the reference sizes it (renderer.ts:405-409).
uint32_t aoExtent(float viewport, float scale);
cudaError_t launchGtao(HfbCtx* c, const HfbUniforms& u, const float* depth, const float* normals, float scale,
                       float* ao);
cudaError_t launchPresent(HfbCtx* c, const HfbUniforms& u, uint32_t W, uint32_t H, const float* result,
                          const float* scene, uint8_t* rgba);
cudaError_t launchPresentBatch(HfbCtx* c, const HfbPresentItem* items, uint32_t n);
// The hair depth pass's list of big triangles has its own region of the
// raster scratch, after the tiles and fine passes' working memory, so the
// pass can run beside them: HD_LIST_ENTRIES entries + the count.
constexpr size_t HD_LIST_ENTRIES = 65536;
inline size_t rasterPassScratchBytes(const HfbConfig& cfg, uint32_t W, uint32_t H, uint32_t maxDrawn) {
  const size_t t = tilesScratchLayout(nullptr, cfg, W, H, maxDrawn).bytes;
  const size_t f = fineScratchLayout(nullptr, cfg, W, H).bytes;
  return alignUp256(t > f ? t : f);
}
// The list (word 0: count) and its capacity for a scratch buffer; capacity 0
// (every big triangle drawn by its own thread) if the buffer has no room.
inline uint32_t* hairDepthList(void* scratch, size_t scratchBytes, size_t passBytes, uint32_t* cap) {
  if (!scratch || scratchBytes < passBytes + 8u) {
    *cap = 0;
    return nullptr;
  }
  const size_t n = (scratchBytes - passBytes) / 4u - 1u;
  *cap = (uint32_t)(n < HD_LIST_ENTRIES ? n : HD_LIST_ENTRIES);
  return reinterpret_cast<uint32_t*>((char*)scratch + passBytes);
}
// Blocks of the grid splat (GridPostSimPass) over `points` points.
uint32_t gridPostBlocks(uint32_t points);
// Blocks of the hair depth pass over `points` points.
uint32_t hairDepthBlocks(uint32_t points);
// Virtual blocks of kind k for one instance (host side).
uint32_t batchBlocks(const HfbConfig& cfg, BatchKind k, const BatchInst& bi);
// One frame of n checked instances; flips their `current`.  With passMs, the
// passes run as plain launches with an event between them, the call waits,
// and passMs[0..HFB_FRAME_PASSES) receives each pass's GPU time.
cudaError_t frameBatch(HfbCtx* c, HfbInstance* insts, uint32_t n, float* passMs = nullptr);
void frameBatchRelease(HfbCtx* c);

}  // namespace hfb
