// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/hairfb.h"

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
TilesScratch tilesScratchLayout(void* base, const HfbConfig& cfg, uint32_t W, uint32_t H,
                                uint32_t maxDrawn);

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
FineScratch fineScratchLayout(void* base, const HfbConfig& cfg, uint32_t W, uint32_t H);
uint32_t maxDrawnSegments(const HfbConfig& cfg, uint32_t W, uint32_t H);

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

}  // namespace hfb
