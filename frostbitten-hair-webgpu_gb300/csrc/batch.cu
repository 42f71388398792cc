// Whole frames: one pass of one instance (framePass), and hfb_frame_batch's
// frame of many instances on worker streams.
//
// A batched frame runs each instance's own pass sequence -- the same
// launches as hfb_frame -- on one of BATCH_STREAMS worker streams forked from
// the context's stream and joined back into it.  Instances share no device
// buffer (the device counters take atomics only), so the streams run their
// instances' kernels side by side: the small launches of a small instance
// (the one-CTA tile sort and fine schedule, a tiles raster of a few hundred
// blocks) fill the SMs another instance leaves idle.  Instances go to the
// stream with the least work so far, largest first.
#include <algorithm>
#include <numeric>
#include <vector>

#define HFB_TU 5
#include "hfb_internal.cuh"

namespace hfb {

static_assert(BATCH_STREAMS == sizeof(HfbCtx::batchStreams) / sizeof(cudaStream_t), "stream table size");

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
      return launchGridPostSim(c, su, h, now, prev, in->densityVelocity);
    case FP_CLEAR:
      return clearRaster(c, rb);
    case FP_TILES:
      return launchTilesPass(c, u, h, prev, in->tangents, in->sceneDepth, in->strandsToRender, rb);
    case FP_SORT:
      return launchTileSort(c, rb);
    case FP_FINE:
      return launchFinePass(c, u, h, prev, in->tangents, in->shading, in->sceneDepth, rb);
    case FP_SHADING:
      if (!h.strandsCount) return cudaSuccess;
      return launchShading(c, u, h, prev, in->tangents, in->shadingDepth ? in->shadingDepth : in->sceneDepth,
                           in->ao, in->ao ? in->aoWidth : 0u, in->ao ? in->aoHeight : 0u, in->shadowMap,
                           in->shadowMap ? in->shadowMapSize : 0u, in->shading);
    default:
      return cudaErrorInvalidValue;
  }
}

namespace {

// Rough GPU work of one instance's frame, for balancing the streams: the
// per-point passes and the per-pixel passes.
double frameWork(const HfbInstance& in) {
  return (double)in.hair.strandsCount * in.hair.pointsPerStrand +
         0.25 * (double)in.raster.width * in.raster.height;
}

cudaError_t ensureStreams(HfbCtx* c) {
  cudaError_t e = cudaSuccess;
  if (!c->batchFork) e = cudaEventCreateWithFlags(&c->batchFork, cudaEventDisableTiming);
  for (uint32_t s = 0; s < BATCH_STREAMS && e == cudaSuccess; s++) {
    if (!c->batchStreams[s]) e = cudaStreamCreateWithFlags(&c->batchStreams[s], cudaStreamNonBlocking);
    if (e == cudaSuccess && !c->batchJoin[s]) e = cudaEventCreateWithFlags(&c->batchJoin[s], cudaEventDisableTiming);
  }
  return e;
}

// Pass by pass over all instances on c->stream, an event between passes.
cudaError_t frameBatchProfiled(HfbCtx* c, HfbInstance* insts, uint32_t n, float* passMs) {
  cudaEvent_t ev[FP_COUNT + 1] = {};
  cudaError_t e = cudaSuccess;
  for (uint32_t i = 0; i <= FP_COUNT && e == cudaSuccess; i++) e = cudaEventCreate(&ev[i]);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], c->stream);
  for (uint32_t p = 0; p < FP_COUNT && e == cudaSuccess; p++) {
    for (uint32_t i = 0; i < n && e == cudaSuccess; i++) e = framePass(c, &insts[i], (FramePass)p);
    if (e == cudaSuccess) e = cudaEventRecord(ev[p + 1], c->stream);
  }
  if (e == cudaSuccess) e = cudaEventSynchronize(ev[FP_COUNT]);
  for (uint32_t p = 0; p < FP_COUNT && e == cudaSuccess; p++) e = cudaEventElapsedTime(&passMs[p], ev[p], ev[p + 1]);
  for (uint32_t i = 0; i <= FP_COUNT; i++)
    if (ev[i]) cudaEventDestroy(ev[i]);
  return e;
}

}  // namespace

cudaError_t frameBatch(HfbCtx* c, HfbInstance* insts, uint32_t n, float* passMs) {
  cudaError_t e = cudaSuccess;
  if (passMs) {
    e = frameBatchProfiled(c, insts, n, passMs);
  } else {
    e = ensureStreams(c);
    if (e != cudaSuccess) return e;
    const uint32_t K = n < BATCH_STREAMS ? n : BATCH_STREAMS;
    // largest instance first, each onto the least-loaded stream
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return frameWork(insts[a]) > frameWork(insts[b]); });
    double load[BATCH_STREAMS] = {};
    e = cudaEventRecord(c->batchFork, c->stream);
    for (uint32_t s = 0; s < K && e == cudaSuccess; s++) e = cudaStreamWaitEvent(c->batchStreams[s], c->batchFork, 0);
    if (e != cudaSuccess) return e;
    const cudaStream_t caller = c->stream;
    for (uint32_t k = 0; k < n && e == cudaSuccess; k++) {
      const uint32_t i = order[k];
      const uint32_t s = (uint32_t)(std::min_element(load, load + K) - load);
      load[s] += frameWork(insts[i]);
      c->stream = c->batchStreams[s];
      for (uint32_t p = 0; p < FP_COUNT && e == cudaSuccess; p++) e = framePass(c, &insts[i], (FramePass)p);
    }
    c->stream = caller;
    // join every worker stream back into the caller's stream, also after a failed launch
    for (uint32_t s = 0; s < K; s++) {
      cudaError_t ej = cudaEventRecord(c->batchJoin[s], c->batchStreams[s]);
      if (ej == cudaSuccess) ej = cudaStreamWaitEvent(caller, c->batchJoin[s], 0);
      if (e == cudaSuccess) e = ej;
    }
  }
  if (e != cudaSuccess) return e;
  for (uint32_t i = 0; i < n; i++) insts[i].current ^= 1u;
  return cudaGetLastError();
}

void frameBatchRelease(HfbCtx* c) {
  for (uint32_t s = 0; s < BATCH_STREAMS; s++) {
    if (c->batchJoin[s]) cudaEventDestroy(c->batchJoin[s]);
    if (c->batchStreams[s]) cudaStreamDestroy(c->batchStreams[s]);
    c->batchJoin[s] = nullptr;
    c->batchStreams[s] = nullptr;
  }
  if (c->batchFork) cudaEventDestroy(c->batchFork);
  c->batchFork = nullptr;
}

}  // namespace hfb
