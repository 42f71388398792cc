// C-ABI of libhairfb.so: context, buffers, validation and the pass entry
// points declared in include/hairfb.h.  Every entry point converts CUDA and
// argument errors into HFB_ERR_* codes plus a message; nothing throws across
// the boundary.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <utility>
#include <vector>

#define HFB_TU 4
#include "hfb_internal.cuh"

namespace {

int fail(HfbCtx* c, int code, const std::string& msg) {
  if (c) c->lastError = msg;
  return code;
}

int cudaFail(HfbCtx* c, cudaError_t e, const char* what) {
  return fail(c, HFB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define HFB_CHECK_CTX(c)                                     \
  do {                                                       \
    if (!(c)) return HFB_ERR_INVALID_ARGUMENT;               \
  } while (0)

#define HFB_REQUIRE(c, cond, msg)                                   \
  do {                                                              \
    if (!(cond)) return fail((c), HFB_ERR_INVALID_ARGUMENT, (msg)); \
  } while (0)

#define HFB_LAUNCH(c, expr, what)                       \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cudaFail((c), e_, (what)); \
    return HFB_OK;                                      \
  } while (0)

bool isPow2(uint32_t v) { return v && !(v & (v - 1u)); }

std::string validateConfig(const HfbConfig& c) {
  if (c.tileSize != 8 && c.tileSize != 16 && c.tileSize != 32) return "tileSize must be 8, 16 or 32";
  if (c.tileDepthBins < 1 || c.tileDepthBins > 64) return "tileDepthBins must be in [1, 64]";
  if (c.slicesPerPixel < 1 || c.slicesPerPixel > 16) return "slicesPerPixel must be in [1, 16]";
  if (c.tileSize == 32 && c.slicesPerPixel > 8) return "32x32 tiles support at most 8 slices";
  if (c.shadingPoints < 2 || c.shadingPoints > 1024) return "shadingPoints must be in [2, 1024]";
  if (c.gridDims < 2 || c.gridDims > 512) return "gridDims must be in [2, 512]";
  if (c.sortBuckets < 1 || c.sortBuckets > 256) return "sortBuckets must be in [1, 256]";
  if (c.sortBucketSize < 1) return "sortBucketSize must be >= 1";
  if (c.avgFragmentsPerSlice < 1) return "avgFragmentsPerSlice must be >= 1";
  if (!(c.alphaMultiplier == c.alphaMultiplier)) return "alphaMultiplier is NaN";
  if (!(c.cameraNear > 0.0f) || !(c.cameraFar > c.cameraNear)) return "camera near/far invalid";
  (void)isPow2;
  return "";
}

std::string validateHair(const HfbHairData* h, uint32_t minPoints = 2, uint32_t maxPoints = 256) {
  if (!h) return "hair data is NULL";
  if (h->pointsPerStrand < minPoints || h->pointsPerStrand > maxPoints)
    return "pointsPerStrand must be in [" + std::to_string(minPoints) + ", " + std::to_string(maxPoints) + "]";
  if (h->strandsCount >= (1u << 24)) return "strandsCount must be < 2^24 (segment encoding)";
  return "";
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

namespace hfb {

uint32_t maxDrawnSegments(const HfbConfig& cfg, uint32_t W, uint32_t H) {
  uint64_t t = (uint64_t)divCeil(W, cfg.tileSize) * divCeil(H, cfg.tileSize);
  return (uint32_t)(1ull + t * cfg.avgSegmentsPerTile);
}

}  // namespace hfb

extern "C" {

int hfb_version(void) { return HFB_VERSION; }

int hfb_ctx_create(const HfbConfig* cfg, int device, HfbCtx** out) {
  if (!cfg || !out) return HFB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::string err = validateConfig(*cfg);
  if (!err.empty()) {
    fprintf(stderr, "hairfb: invalid config: %s\n", err.c_str());
    return HFB_ERR_INVALID_ARGUMENT;
  }
  HfbCtx* c = new (std::nothrow) HfbCtx();
  if (!c) return HFB_ERR_OUT_OF_MEMORY;
  c->cfg = *cfg;
  cudaError_t e;
  if (device >= 0) {
    e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete c; return HFB_ERR_CUDA; }
  }
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->smCount, cudaDevAttrMultiProcessorCount, c->device);
  e = cudaStreamCreateWithFlags(&c->ownStream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return HFB_ERR_CUDA; }
  c->stream = c->ownStream;
  e = cudaMalloc(&c->dCounters, sizeof(hfb::DeviceCounters));
  if (e != cudaSuccess) { cudaStreamDestroy(c->ownStream); delete c; return HFB_ERR_OUT_OF_MEMORY; }
  cudaMemsetAsync(c->dCounters, 0, sizeof(hfb::DeviceCounters), c->stream);
  cudaStreamSynchronize(c->stream);
  hfb::noallocPrepare(c);
  *out = c;
  return HFB_OK;
}

int hfb_ctx_destroy(HfbCtx* c) {
  HFB_CHECK_CTX(c);
  cudaStreamSynchronize(c->stream);
  hfb::frameBatchRelease(c);
  if (c->checkDev) cudaFree(c->checkDev);
  if (c->dCounters) cudaFree(c->dCounters);
  if (c->ownStream) cudaStreamDestroy(c->ownStream);
  delete c;
  return HFB_OK;
}

const char* hfb_last_error(const HfbCtx* c) { return c ? c->lastError.c_str() : "null context"; }

int hfb_ctx_set_stream(HfbCtx* c, void* stream) {
  HFB_CHECK_CTX(c);
  c->stream = stream ? (cudaStream_t)stream : c->ownStream;
  return HFB_OK;
}

int hfb_sync(HfbCtx* c) {
  HFB_CHECK_CTX(c);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cudaFail(c, e, "hfb_sync");
  return HFB_OK;
}

int hfb_get_counters(HfbCtx* c, HfbCounters* out) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, out, "out is NULL");
  hfb::DeviceCounters d;
  cudaError_t e = cudaMemcpyAsync(&d, c->dCounters, sizeof(d), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cudaFail(c, e, "hfb_get_counters");
  memset(out, 0, sizeof(*out));
  out->tileRecords = d.tileRecords;
  out->tileRecordsDropped = d.tileRecordsDropped;
  out->finePoolFullBins = d.finePoolFullBins;
  out->launches = c->launches;
  out->fineSplitTiles = d.fineSplitTiles;
  out->fineSplitRedone = d.fineSplitRedone;
  out->badWorkItems = d.badWorkItems;
  return HFB_OK;
}

int hfb_check_constant_division(HfbCtx* c, uint64_t out[3]) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, out, "out is NULL");
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMalloc(&d, 3 * sizeof(unsigned long long));
  if (e != cudaSuccess) return cudaFail(c, e, "hfb_check_constant_division");
  unsigned long long h[3] = {0, 0, 0};
  e = hfb::launchConstDivCheck(c, d);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (e != cudaSuccess) return cudaFail(c, e, "hfb_check_constant_division");
  for (int i = 0; i < 3; i++) out[i] = h[i];
  return HFB_OK;
}

int hfb_buffer_alloc(HfbCtx* c, size_t bytes, void** out) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, out, "out is NULL");
  *out = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(c, HFB_ERR_OUT_OF_MEMORY, "cudaMalloc failed: " + std::string(cudaGetErrorString(e)));
  }
  return HFB_OK;
}

int hfb_buffer_free(HfbCtx* c, void* ptr) {
  HFB_CHECK_CTX(c);
  if (!ptr) return HFB_OK;
  cudaStreamSynchronize(c->stream);
  cudaError_t e = cudaFree(ptr);
  if (e != cudaSuccess) return cudaFail(c, e, "cudaFree");
  return HFB_OK;
}

int hfb_buffer_upload(HfbCtx* c, void* dst, const void* src, size_t bytes) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, dst && src, "NULL pointer");
  HFB_LAUNCH(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream), "upload");
}

int hfb_buffer_download(HfbCtx* c, void* dst, const void* src, size_t bytes) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, dst && src, "NULL pointer");
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cudaFail(c, e, "download");
  return HFB_OK;
}

int hfb_buffer_clear(HfbCtx* c, void* dst, size_t bytes) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, dst, "NULL pointer");
  HFB_LAUNCH(c, cudaMemsetAsync(dst, 0, bytes, c->stream), "clear");
}

size_t hfb_raster_scratch_bytes_for(const HfbConfig* cfg, uint32_t width, uint32_t height, uint32_t maxDrawn) {
  if (!cfg || width == 0 || height == 0 || maxDrawn == 0) return 0;
  return hfb::rasterPassScratchBytes(*cfg, width, height, maxDrawn) + (hfb::HD_LIST_ENTRIES + 1u) * 4u;
}

size_t hfb_raster_scratch_bytes(const HfbConfig* cfg, uint32_t width, uint32_t height) {
  if (!cfg || width == 0 || height == 0) return 0;
  return hfb_raster_scratch_bytes_for(cfg, width, height, hfb::maxDrawnSegments(*cfg, width, height));
}

int hfb_raster_buffers_alloc_sized(HfbCtx* c, uint32_t W, uint32_t H, uint32_t maxDrawn, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, rb, "rb is NULL");
  HFB_REQUIRE(c, W > 0 && H > 0 && W <= 16384 && H <= 16384, "viewport must be 1..16384 px");
  HFB_REQUIRE(c, maxDrawn >= 1 && maxDrawn < 0xFFFFFFF0u, "maxDrawnSegments must be in [1, 2^32 - 16)");
  memset(rb, 0, sizeof(*rb));
  const HfbConfig& cfg = c->cfg;
  size_t T = (size_t)hfb::divCeil(W, cfg.tileSize) * hfb::divCeil(H, cfg.tileSize);
  const uint64_t md = maxDrawn;
  rb->width = W;
  rb->height = H;
  rb->maxDrawnSegments = (uint32_t)md;
  struct { void** p; size_t bytes; } req[] = {
      {(void**)&rb->tiles, T * cfg.tileDepthBins * 16},
      {(void**)&rb->tileSegments, 4 + (size_t)md * 8},
      {(void**)&rb->segmentCountPerTile, T * 4},
      {(void**)&rb->sortBuckets, (size_t)cfg.sortBuckets * 8},
      {(void**)&rb->tileList, (4 + T) * 4},
      {(void**)&rb->rasterizerResult, 16 + (size_t)W * H * 16},
  };
  for (auto& r : req) {
    if (cudaMalloc(r.p, r.bytes) != cudaSuccess) {
      cudaGetLastError();
      hfb_raster_buffers_free(c, rb);
      return fail(c, HFB_ERR_OUT_OF_MEMORY, "raster buffer allocation failed");
    }
  }
  rb->scratchBytes = hfb_raster_scratch_bytes_for(&cfg, W, H, (uint32_t)md);
  if (cudaMalloc(&rb->scratch, rb->scratchBytes) != cudaSuccess) {
    cudaGetLastError();
    hfb_raster_buffers_free(c, rb);
    return fail(c, HFB_ERR_OUT_OF_MEMORY, "raster scratch allocation failed");
  }
  cudaMemsetAsync(rb->scratch, 0, rb->scratchBytes, c->stream);
  return hfb_clear_before_render(c, rb);
}

int hfb_raster_buffers_alloc(HfbCtx* c, uint32_t W, uint32_t H, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, W > 0 && H > 0 && W <= 16384 && H <= 16384, "viewport must be 1..16384 px");
  const uint64_t T = (uint64_t)hfb::divCeil(W, c->cfg.tileSize) * hfb::divCeil(H, c->cfg.tileSize);
  const uint64_t md = 1ull + T * c->cfg.avgSegmentsPerTile;
  HFB_REQUIRE(c, md < 0xFFFFFFF0ull, "maxDrawnHairSegments overflows u32");
  return hfb_raster_buffers_alloc_sized(c, W, H, (uint32_t)md, rb);
}

int hfb_raster_buffers_free(HfbCtx* c, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  if (!rb) return HFB_OK;
  cudaStreamSynchronize(c->stream);
  void* ps[] = {rb->tiles, rb->tileSegments, rb->segmentCountPerTile, rb->sortBuckets,
                rb->tileList, rb->rasterizerResult, rb->scratch};
  for (void* p : ps)
    if (p) cudaFree(p);
  memset(rb, 0, sizeof(*rb));
  return HFB_OK;
}

static std::string checkRaster(const HfbCtx* c, const HfbRasterBuffers* rb) {
  if (!rb) return "raster buffers are NULL";
  if (!rb->tiles || !rb->tileSegments || !rb->segmentCountPerTile || !rb->sortBuckets ||
      !rb->tileList || !rb->rasterizerResult || !rb->scratch)
    return "a raster buffer is NULL";
  if (rb->width == 0 || rb->height == 0) return "raster buffers have an empty viewport";
  if (rb->maxDrawnSegments == 0) return "maxDrawnSegments is 0";
  if (rb->scratchBytes < hfb_raster_scratch_bytes_for(&c->cfg, rb->width, rb->height, rb->maxDrawnSegments))
    return "raster scratch is too small";
  return "";
}

static std::string checkViewport(const HfbUniforms* u, const HfbRasterBuffers* rb) {
  if (!u) return "uniforms are NULL";
  if (!(u->viewport.x == (float)rb->width) || !(u->viewport.y == (float)rb->height))
    return "Uniforms.viewport does not match the raster buffers";
  if (u->maxDrawnHairSegments != rb->maxDrawnSegments)
    return "Uniforms.maxDrawnHairSegments does not match the raster buffers";
  return "";
}

int hfb_clear_before_render(HfbCtx* c, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  std::string err = checkRaster(c, rb);
  HFB_REQUIRE(c, err.empty(), err);
  cudaError_t e = hfb::clearRaster(c, *rb);
  if (e != cudaSuccess) return cudaFail(c, e, "clear_before_render");
  return HFB_OK;
}

int hfb_grid_pre_sim(HfbCtx* c, const HfbSimUniforms* u, const int32_t* dv, float* gw, const float* sdf,
                     uint32_t sdfDims) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && dv && gw && sdf, "NULL argument");
  HFB_REQUIRE(c, sdfDims >= 1 && sdfDims <= 1024, "sdfDims must be in [1, 1024]");
  HFB_REQUIRE(c, aligned16(dv) && aligned16(gw), "grid buffers must be 16-byte aligned");
  HFB_LAUNCH(c, hfb::launchGridPreSim(c, *u, dv, gw, sdf, sdfDims), "grid_pre_sim");
}

int hfb_sim_integrate(HfbCtx* c, const HfbSimUniforms* u, const HfbHairData* h, float* prev,
                      const float* now, const float* initial, const float* segLen, const int32_t* dv,
                      const float* gw, const float* sdf, uint32_t sdfDims) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && prev && now && initial && segLen && dv && gw && sdf, "NULL argument");
  // the local shape constraint needs >= 4 points; a strand must fit the
  // block's shared-memory staging (128 points x 64 strands x 16 B)
  std::string err = validateHair(h, 4, 128);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_REQUIRE(c, sdfDims >= 1 && sdfDims <= 1024, "sdfDims must be in [1, 1024]");
  HFB_REQUIRE(c, u->constraintIterations <= 1024, "constraintIterations must be <= 1024");
  HFB_REQUIRE(c, aligned16(prev) && aligned16(now) && aligned16(initial) && aligned16(dv) && aligned16(gw),
              "vec4 buffers must be 16-byte aligned");
  if (h->strandsCount == 0) return HFB_OK;
  HFB_LAUNCH(c, hfb::launchSimIntegrate(c, *u, *h, prev, now, initial, segLen, dv, gw, sdf, sdfDims),
             "sim_integrate");
}

int hfb_grid_post_sim(HfbCtx* c, const HfbSimUniforms* u, const HfbHairData* h, const float* prev,
                      const float* now, int32_t* dv) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && prev && now && dv, "NULL argument");
  std::string err = validateHair(h);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_REQUIRE(c, aligned16(prev) && aligned16(now) && aligned16(dv), "vec4 buffers must be 16-byte aligned");
  HFB_LAUNCH(c, hfb::launchGridPostSim(c, *u, *h, prev, now, dv, nullptr), "grid_post_sim");
}

int hfb_grid_post_sim_ordered(HfbCtx* c, const HfbSimUniforms* u, const HfbHairData* h, const float* prev,
                              const float* now, int32_t* dv, const uint32_t* order) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && prev && now && dv, "NULL argument");
  std::string err = validateHair(h);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_REQUIRE(c, aligned16(prev) && aligned16(now) && aligned16(dv), "vec4 buffers must be 16-byte aligned");
  HFB_LAUNCH(c, hfb::launchGridPostSim(c, *u, *h, prev, now, dv, order), "grid_post_sim");
}

namespace {
// Bits 0..9 of v spread to every third bit.
uint64_t mortonSpread(uint32_t v) {
  uint64_t x = v & 0x3ffu;
  x = (x | (x << 16)) & 0x030000FFull;
  x = (x | (x << 8)) & 0x0300F00Full;
  x = (x | (x << 4)) & 0x030C30C3ull;
  x = (x | (x << 2)) & 0x09249249ull;
  return x;
}
}  // namespace

int hfb_strand_grid_order(const float* pos, uint32_t S, uint32_t P, uint32_t* out) {
  if (!out || (S && (!pos || P == 0))) return HFB_ERR_INVALID_ARGUMENT;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t s = 0; s < S; s++)
    for (int a = 0; a < 3; a++) {
      const float v = pos[(size_t)s * P * 4 + a];
      if (std::isfinite(v)) {
        lo[a] = std::min(lo[a], v);
        hi[a] = std::max(hi[a], v);
      }
    }
  std::vector<std::pair<uint64_t, uint32_t>> keys(S);
  for (uint32_t s = 0; s < S; s++) {
    uint64_t code = 0;
    for (int a = 0; a < 3; a++) {
      const float v = pos[(size_t)s * P * 4 + a];
      const double ext = (double)hi[a] - (double)lo[a];
      double t = std::isfinite(v) && ext > 0.0 ? ((double)v - (double)lo[a]) / ext : 0.0;
      t = std::min(std::max(t, 0.0), 1.0);
      code |= mortonSpread((uint32_t)(t * 1023.0)) << a;
    }
    keys[s] = {code, s};
  }
  std::stable_sort(keys.begin(), keys.end(),
                   [](const std::pair<uint64_t, uint32_t>& x, const std::pair<uint64_t, uint32_t>& y) {
                     return x.first < y.first;
                   });
  for (uint32_t s = 0; s < S; s++) out[s] = keys[s].second;
  return HFB_OK;
}

int hfb_shading(HfbCtx* c, const HfbUniforms* u, const HfbHairData* h, const float* pos,
                const float* tan, const float* depth, const float* ao, uint32_t aoW, uint32_t aoH,
                const float* sm, uint32_t smSize, float* shading) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && pos && tan && depth && shading, "NULL argument");
  std::string err = validateHair(h);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_REQUIRE(c, !ao || (aoW > 0 && aoH > 0), "AO texture with an empty size");
  HFB_REQUIRE(c, !sm || smSize > 0, "shadow map with an empty size");
  HFB_REQUIRE(c, u->viewport.x >= 1.0f && u->viewport.y >= 1.0f, "viewport is empty");
  HFB_REQUIRE(c, aligned16(pos) && aligned16(tan) && aligned16(shading), "vec4 buffers must be 16-byte aligned");
  if (h->strandsCount == 0) return HFB_OK;
  HFB_LAUNCH(c, hfb::launchShading(c, *u, *h, pos, tan, depth, ao, aoW, aoH, sm, smSize, shading),
             "shading");
}

int hfb_tiles_pass(HfbCtx* c, const HfbUniforms* u, const HfbHairData* h, const float* pos,
                   const float* tan, const float* depth, uint32_t strandsToRender, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, pos && tan && depth, "NULL argument");
  HFB_REQUIRE(c, aligned16(pos) && aligned16(tan), "vec4 buffers must be 16-byte aligned");
  std::string err = validateHair(h);
  if (err.empty()) err = checkRaster(c, rb);
  if (err.empty()) err = checkViewport(u, rb);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_LAUNCH(c, hfb::launchTilesPass(c, *u, *h, pos, tan, depth, strandsToRender, *rb), "tiles_pass");
}

int hfb_tile_sort(HfbCtx* c, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  std::string err = checkRaster(c, rb);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_LAUNCH(c, hfb::launchTileSort(c, *rb), "tile_sort");
}

int hfb_fine_pass(HfbCtx* c, const HfbUniforms* u, const HfbHairData* h, const float* pos,
                  const float* tan, const float* shading, const float* depth, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, pos && tan && shading && depth, "NULL argument");
  HFB_REQUIRE(c, aligned16(pos) && aligned16(tan) && aligned16(shading), "vec4 buffers must be 16-byte aligned");
  std::string err = validateHair(h);
  if (err.empty()) err = checkRaster(c, rb);
  if (err.empty()) err = checkViewport(u, rb);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_LAUNCH(c, hfb::launchFinePass(c, *u, *h, pos, tan, shading, depth, *rb), "fine_pass");
}

int hfb_hair_depth(HfbCtx* c, const HfbUniforms* u, const HfbHairData* h, const float* pos, const float* tan,
                   uint32_t strandsToRender, const float* sceneDepth, float* hairDepth, HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, pos && tan && sceneDepth && hairDepth, "NULL argument");
  HFB_REQUIRE(c, aligned16(pos) && aligned16(tan), "vec4 buffers must be 16-byte aligned");
  std::string err = validateHair(h);
  if (err.empty()) err = checkRaster(c, rb);
  if (err.empty()) err = checkViewport(u, rb);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_LAUNCH(c, hfb::launchHairDepth(c, *u, *h, pos, tan, strandsToRender, sceneDepth, hairDepth, *rb), "hair_depth");
}

int hfb_hair_normals(HfbCtx* c, const HfbUniforms* u, const HfbHairData* h, const float* pos, const float* tan,
                     uint32_t strandsToRender, const float* hairDepth, float* normals, uint32_t* winner,
                     HfbRasterBuffers* rb) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && pos && tan && hairDepth && normals && winner, "NULL argument");
  HFB_REQUIRE(c, aligned16(pos) && aligned16(tan), "vec4 buffers must be 16-byte aligned");
  std::string err = validateHair(h);
  if (err.empty()) err = checkRaster(c, rb);
  if (err.empty()) err = checkViewport(u, rb);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_LAUNCH(c, hfb::launchHairNormals(c, *u, *h, pos, tan, strandsToRender, hairDepth, normals, winner, *rb),
             "hair_normals");
}

int hfb_gtao(HfbCtx* c, const HfbUniforms* u, const float* depth, const float* normals, float scale, float* ao) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && depth && normals && ao, "NULL argument");
  HFB_REQUIRE(c, scale > 0.0f && scale <= 1.0f, "scale must be in (0, 1]");
  HFB_REQUIRE(c, u->viewport.x >= 1.0f && u->viewport.y >= 1.0f && u->viewport.x <= 65536.0f &&
                     u->viewport.y <= 65536.0f, "the viewport must be in [1, 65536]");
  HFB_REQUIRE(c, u->ao.numDirections <= 64 && u->ao.numSteps <= 64, "numDirections and numSteps must be <= 64");
  HFB_LAUNCH(c, hfb::launchGtao(c, *u, depth, normals, scale, ao), "gtao");
}

int hfb_present(HfbCtx* c, const HfbUniforms* u, const HfbRasterBuffers* rb, const float* scene, uint8_t* rgba) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, u && rgba, "NULL argument");
  HFB_REQUIRE(c, !scene || aligned16(scene), "vec4 buffers must be 16-byte aligned");
  std::string err = checkRaster(c, rb);
  if (err.empty()) err = checkViewport(u, rb);
  HFB_REQUIRE(c, err.empty(), err);
  HFB_LAUNCH(c, hfb::launchPresent(c, *u, rb->width, rb->height, rb->rasterizerResult + 4, scene, rgba), "present");
}

int hfb_present_batch(HfbCtx* c, const HfbPresentItem* items, uint32_t n) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, n == 0 || items, "NULL argument");
  for (uint32_t k = 0; k < n; k++) {
    const HfbPresentItem& it = items[k];
    const std::string at = "item " + std::to_string(k) + ": ";
    HFB_REQUIRE(c, it.uniforms && it.rgba, at + "NULL argument");
    HFB_REQUIRE(c, !it.sceneColor || aligned16(it.sceneColor), at + "vec4 buffers must be 16-byte aligned");
    std::string err = checkRaster(c, it.rb);
    if (err.empty()) err = checkViewport(it.uniforms, it.rb);
    HFB_REQUIRE(c, err.empty(), at + err);
  }
  HFB_LAUNCH(c, hfb::launchPresentBatch(c, items, n), "present_batch");
}

// Checks one instance of a frame (the union of the per-pass checks).
static std::string checkInstance(const HfbCtx* c, const HfbInstance* in) {
  if (!in) return "instance is NULL";
  if (!in->uniforms || !in->simUniforms) return "instance uniforms are NULL";
  std::string err = validateHair(&in->hair, 4, 128);
  if (!err.empty()) return err;
  if (!in->positions[0] || !in->positions[1] || !in->positionsInitial || !in->tangents || !in->segmentLengths ||
      !in->densityVelocity || !in->densityGradWind || !in->sdf || !in->shading || !in->sceneDepth)
    return "an instance buffer is NULL";
  if (in->positions[0] == in->positions[1]) return "the two position buffers are the same";
  if (in->current > 1u) return "current must be 0 or 1";
  if (!aligned16(in->positions[0]) || !aligned16(in->positions[1]) || !aligned16(in->positionsInitial) ||
      !aligned16(in->tangents) || !aligned16(in->densityVelocity) || !aligned16(in->densityGradWind) ||
      !aligned16(in->shading))
    return "vec4 buffers must be 16-byte aligned";
  if (in->sdfDims < 1 || in->sdfDims > 1024) return "sdfDims must be in [1, 1024]";
  if (in->simUniforms->constraintIterations > 1024) return "constraintIterations must be <= 1024";
  if (in->ao && (in->aoWidth == 0 || in->aoHeight == 0)) return "AO texture with an empty size";
  if (in->shadowMap && in->shadowMapSize == 0) return "shadow map with an empty size";
  err = checkRaster(c, &in->raster);
  if (err.empty()) err = checkViewport(in->uniforms, &in->raster);
  return err;
}

int hfb_frame(HfbCtx* c, HfbInstance* in) {
  HFB_CHECK_CTX(c);
  std::string err = checkInstance(c, in);
  HFB_REQUIRE(c, err.empty(), err);
  cudaError_t e = cudaSuccess;
  for (uint32_t p = 0; p < hfb::FP_COUNT && e == cudaSuccess; p++) e = hfb::framePass(c, in, (hfb::FramePass)p);
  if (e != cudaSuccess) return cudaFail(c, e, "frame");
  in->current ^= 1u;
  return HFB_OK;
}

int hfb_frame_batch(HfbCtx* c, HfbInstance* insts, uint32_t n) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, insts || n == 0, "instances are NULL");
  HFB_REQUIRE(c, n <= hfb::BATCH_MAX, "at most 1024 instances per batch");
  if (n == 0) return HFB_OK;
  for (uint32_t i = 0; i < n; i++) {
    std::string err = checkInstance(c, &insts[i]);
    HFB_REQUIRE(c, err.empty(), "instance " + std::to_string(i) + ": " + err);
  }
  cudaError_t e = hfb::frameBatch(c, insts, n);
  if (e != cudaSuccess) return cudaFail(c, e, "frame_batch");
  return HFB_OK;
}

int hfb_ctx_set_batch_groups(HfbCtx* c, uint32_t groups) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, groups >= 1 && groups <= hfb::BATCH_GROUPS_MAX, "batch groups must be in [1, 4]");
  c->batchGroups = groups;
  return HFB_OK;
}

int hfb_ctx_set_batch_pipeline(HfbCtx* c, uint32_t on) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, on <= 1u, "pipeline must be 0 or 1");
  if ((on != 0u) != c->batchPipeline) {  // a clean start: nothing of the other mode in flight
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cudaFail(c, e, "ctx_set_batch_pipeline");
    c->batchPipeline = on != 0u;
    c->pipeCalls = 0;
  }
  return HFB_OK;
}

int hfb_frame_batch_profile(HfbCtx* c, HfbInstance* insts, uint32_t n, float* passMs) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, insts && n > 0 && passMs, "NULL argument or empty batch");
  HFB_REQUIRE(c, n <= hfb::BATCH_MAX, "at most 1024 instances per batch");
  for (uint32_t i = 0; i < n; i++) {
    std::string err = checkInstance(c, &insts[i]);
    HFB_REQUIRE(c, err.empty(), "instance " + std::to_string(i) + ": " + err);
  }
  cudaError_t e = hfb::frameBatch(c, insts, n, passMs);
  if (e != cudaSuccess) return cudaFail(c, e, "frame_batch_profile");
  return HFB_OK;
}

#ifdef HFB_DEVICE_CHECKS
// Self-checking build only (not part of include/hairfb.h): registers the
// byte ranges [lo, hi) that the kernels may touch (pairs in lohi; the
// context's own device counters are added), and resets the failure record.
HFB_API int hfb_debug_check_ranges(HfbCtx* c, const unsigned long long* lohi, uint32_t n) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, lohi || n == 0, "NULL ranges");
  HFB_REQUIRE(c, n + 1 <= hfb::CHECK_MAX_RANGES, "too many ranges");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess && !c->checkDev) e = cudaMalloc(&c->checkDev, sizeof(hfb::CheckState));
  if (e != cudaSuccess) return cudaFail(c, e, "debug_check_ranges");
  // sorted by start, duplicates dropped; overlapping ranges are rejected
  std::vector<std::pair<unsigned long long, unsigned long long>> r;
  for (uint32_t i = 0; i < n; i++) r.emplace_back(lohi[2 * i], lohi[2 * i + 1]);
  r.emplace_back((unsigned long long)c->dCounters, (unsigned long long)c->dCounters + sizeof(hfb::DeviceCounters));
  std::sort(r.begin(), r.end());
  r.erase(std::unique(r.begin(), r.end()), r.end());
  for (size_t i = 1; i < r.size(); i++)
    HFB_REQUIRE(c, r[i].first >= r[i - 1].second, "overlapping ranges");
  hfb::CheckState* h = new hfb::CheckState();
  for (size_t i = 0; i < r.size(); i++) {
    h->lo[i] = r[i].first;
    h->hi[i] = r[i].second;
  }
  h->nRanges = (uint32_t)r.size();
  e = cudaMemcpy(c->checkDev, h, sizeof(*h), cudaMemcpyHostToDevice);
  delete h;
  if (e != cudaSuccess) return cudaFail(c, e, "debug_check_ranges");
  return HFB_OK;
}

// out[0] = failed checks, out[1] = translation unit << 16 | line of the
// first, out[2] = its address (0 for a failed condition), out[3] = its bytes.
HFB_API int hfb_debug_check_read(HfbCtx* c, unsigned long long* out) {
  HFB_CHECK_CTX(c);
  HFB_REQUIRE(c, out && c->checkDev, "NULL output or no ranges registered");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  hfb::CheckState h;
  if (e == cudaSuccess) e = cudaMemcpy(&h, c->checkDev, sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cudaFail(c, e, "debug_check_read");
  out[0] = h.fails;
  out[1] = h.firstWhere;
  out[2] = h.firstAddr;
  out[3] = h.firstBytes;
  return HFB_OK;
}
#endif

}  // extern "C"
