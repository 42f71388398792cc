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
  size_t simSmemSet = 0;
  bool largeBinsAttrSet = false;
  int fineBlocksPerSM[3][3] = {};  // [tile 8/16/32][slices 4/8/16]
  // batched frames: worker streams, the fork event and one join event per stream
  cudaStream_t batchStreams[8] = {};
  cudaEvent_t batchFork = nullptr;
  cudaEvent_t batchJoin[8] = {};
  // self-checking build: the device CheckState (hfb_check.cuh), else NULL
  void* checkDev = nullptr;
};

namespace hfb {

// Device counters, mirrored into HfbCounters by hfb_get_counters.
struct DeviceCounters {
  unsigned long long tileRecords;
  unsigned long long tileRecordsDropped;
  unsigned long long finePoolFullBins;
  unsigned long long waitTimeouts;
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

// Strands per integration block for P points per strand: one chain warp per
// block for P <= 32, fewer strands for longer strands (shared memory ~38 KB).
__host__ __device__ inline uint32_t simStrandsPerBlock(uint32_t P) {
  return P <= 32u ? 32u : (1024u / P > 8u ? 1024u / P : 8u);
}
__host__ __device__ inline size_t simSmemBytes(uint32_t P) {
  return (size_t)simStrandsPerBlock(P) * (P + 1u) * (2u * sizeof(float4) + sizeof(float));
}
constexpr uint32_t TILES_RASTER_SEGS = 128;  // segments per tiles-raster block

// Launchers. Each returns cudaSuccess or the launch error.
cudaError_t launchGridPreSim(HfbCtx* c, const HfbSimUniforms& u, const int32_t* dv, float* gw,
                             const float* sdf, uint32_t sdfDims);
cudaError_t launchSimIntegrate(HfbCtx* c, const HfbSimUniforms& u, const HfbHairData& h, float* prev,
                               const float* now, const float* initial, const float* segLen,
                               const int32_t* dv, const float* gw, const float* sdf, uint32_t sdfDims);
cudaError_t launchGridPostSim(HfbCtx* c, const HfbSimUniforms& u, const HfbHairData& h, const float* prev,
                              const float* now, int32_t* dv);
cudaError_t launchShading(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                          const float* tan, const float* depth, const float* ao, uint32_t aoW,
                          uint32_t aoH, const float* sm, uint32_t smSize, float* shading);
cudaError_t launchTilesPass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                            const float* tan, const float* depth, uint32_t strandsToRender,
                            HfbRasterBuffers& rb);
cudaError_t launchTileSort(HfbCtx* c, HfbRasterBuffers& rb);
cudaError_t launchFinePass(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos,
                           const float* tan, const float* shading, const float* depth,
                           HfbRasterBuffers& rb);

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
// Whole frames (hfb_frame, hfb_frame_batch).  A frame of one instance is the
// reference's pass sequence; framePass launches one pass of it on c->stream.
// ---------------------------------------------------------------------------
constexpr uint32_t BATCH_MAX = 1024;   // instances per hfb_frame_batch call
constexpr uint32_t BATCH_STREAMS = 8;  // worker streams of a batched frame
enum FramePass : uint32_t {
  FP_GRID_PRE = 0,  // GridPreSimPass
  FP_INTEGRATE,     // HairSimIntegrationPass
  FP_GRID_POST,     // GridPostSimPass (with its grid clear)
  FP_CLEAR,         // cmdClearBeforeRender of the raster passes
  FP_TILES,         // HairTilesPass
  FP_SORT,          // HairTileSortPass
  FP_FINE,          // HairFinePass
  FP_SHADING,       // HairShadingPass
  FP_COUNT
};
cudaError_t framePass(HfbCtx* c, HfbInstance* in, FramePass p);
cudaError_t clearRaster(HfbCtx* c, const HfbRasterBuffers& rb);
// One frame of n checked instances on the worker streams (instance i on
// stream i mod BATCH_STREAMS), joined back into c->stream; with passMs, the
// passes run pass by pass over all instances on c->stream instead, with an
// event between passes, and passMs[p] receives each pass's GPU time.
// Flips every instance's `current`.
cudaError_t frameBatch(HfbCtx* c, HfbInstance* insts, uint32_t n, float* passMs = nullptr);
void frameBatchRelease(HfbCtx* c);

}  // namespace hfb
