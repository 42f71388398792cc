// hfb_tiles_pass_noalloc: the tiles pass for callers that cannot allocate
// device memory.
//
// Some hosts cannot call cudaMalloc when they need to bin a frame: a
// real-time render thread that must not take the device-wide
// synchronisation cudaMalloc may imply, a host whose allocator owns every
// device byte and forbids driver allocations after start-up, or code that is
// about to record its work into a stream capture.  hfb_tiles_pass needs
// working memory (per-bin counts and offsets, record keys, scan partials)
// that normally lives in HfbRasterBuffers.scratch, allocated by the caller or
// by hfb_raster_buffers_alloc.  This entry point takes that working memory
// from one fixed array compiled into the library instead.
//
// Facts a caller relies on:
//   - the array holds HFB_NOALLOC_SCRATCH_BYTES (16 MiB); a viewport whose
//     tiles pass needs more (hfb_raster_scratch_bytes) is rejected with
//     HFB_ERR_INVALID_ARGUMENT and a message, before any work is queued;
//   - every GPU that loads the library holds the array until the process
//     exits;
//   - every call shares the one array, which keeps the last call's contents:
//     the pass zeroes what must start at zero on every call, and two calls
//     whose work overlaps on the GPU (different streams or contexts on the
//     same device, without ordering between them) race on the array;
//   - the array's device address is looked up when a context is created
//     (hfb_ctx_create, with the context's device current, through
//     cudaGetSymbolAddress) and kept in the context.  CUDA loads a
//     library's device code lazily, one source file at a time, so that
//     lookup is also what loads this file's code onto the device and
//     allocates the array: it happens once per device, inside
//     hfb_ctx_create, never inside hfb_tiles_pass_noalloc.  The same set-up
//     loads the tiles pass's kernels (a kernel's first launch would load
//     its code, which takes device memory too).  A context keeps
//     the address for its whole life; a device reset (cudaDeviceReset)
//     invalidates every context anyway, and contexts created after it look
//     the address up again;
//   - the call allocates nothing: no cudaMalloc, no cudaFree, no allocating
//     library routine.  The caller still passes every input and output.
#include <string>

#define HFB_TU 6
#include "hfb_internal.cuh"

namespace {

// The tiles pass's working memory for hfb_tiles_pass_noalloc.
static __device__ __align__(256) unsigned char g_tilesScratch[HFB_NOALLOC_SCRATCH_BYTES];

int fail(HfbCtx* c, int code, const std::string& msg) {
  c->lastError = msg;
  return code;
}

}  // namespace

namespace hfb {

// Set-up at context creation, with the context's device current.
void noallocPrepare(HfbCtx* c) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_tilesScratch);
  // the pass's kernels too: their first launch would otherwise load them
  if (e == cudaSuccess) e = tilesPassLoad(c);
  if (e != cudaSuccess) {
    cudaGetLastError();  // not sticky: the context stays usable for every other pass
    c->noallocScratch = nullptr;
    c->noallocError = std::string("loading the fixed tiles-pass array and the tiles pass's kernels failed when "
                                  "the context was created: ") + cudaGetErrorString(e);
    return;
  }
  c->noallocScratch = p;
  c->noallocError.clear();
}

}  // namespace hfb

namespace {

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

extern "C" HFB_API int hfb_tiles_pass_noalloc(HfbCtx* c, const HfbUniforms* u, const HfbHairData* h,
                                              const float* pos, const float* tan, const float* depth,
                                              uint32_t strandsToRender, HfbRasterBuffers* rb) {
  if (!c) return HFB_ERR_INVALID_ARGUMENT;
  if (!u || !h || !pos || !tan || !depth || !rb) return fail(c, HFB_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!aligned16(pos) || !aligned16(tan)) return fail(c, HFB_ERR_INVALID_ARGUMENT, "vec4 buffers must be 16-byte aligned");
  if (h->pointsPerStrand < 2 || h->pointsPerStrand > 256)
    return fail(c, HFB_ERR_INVALID_ARGUMENT, "pointsPerStrand must be in [2, 256]");
  if (h->strandsCount >= (1u << 24)) return fail(c, HFB_ERR_INVALID_ARGUMENT, "strandsCount must be < 2^24");
  if (!rb->tiles || !rb->tileSegments || !rb->segmentCountPerTile || rb->width == 0 || rb->height == 0)
    return fail(c, HFB_ERR_INVALID_ARGUMENT, "a raster buffer is NULL or the viewport is empty");
  if (rb->maxDrawnSegments == 0) return fail(c, HFB_ERR_INVALID_ARGUMENT, "maxDrawnSegments is 0");
  if (!(u->viewport.x == (float)rb->width) || !(u->viewport.y == (float)rb->height) ||
      u->maxDrawnHairSegments != rb->maxDrawnSegments)
    return fail(c, HFB_ERR_INVALID_ARGUMENT, "Uniforms.viewport / maxDrawnHairSegments do not match the raster buffers");
  const size_t need = hfb_raster_scratch_bytes_for(&c->cfg, rb->width, rb->height, rb->maxDrawnSegments);
  if (need > HFB_NOALLOC_SCRATCH_BYTES)
    return fail(c, HFB_ERR_INVALID_ARGUMENT,
                "the tiles pass needs " + std::to_string(need) + " bytes of working memory for " +
                    std::to_string(rb->width) + "x" + std::to_string(rb->height) +
                    "; the fixed array holds " + std::to_string((size_t)HFB_NOALLOC_SCRATCH_BYTES) +
                    ": use hfb_tiles_pass with HfbRasterBuffers.scratch");
  void* scratch = c->noallocScratch;  // looked up by hfb_ctx_create
  if (!scratch) return fail(c, HFB_ERR_CUDA, c->noallocError);
  HfbRasterBuffers r = *rb;
  r.scratch = scratch;
  r.scratchBytes = HFB_NOALLOC_SCRATCH_BYTES;
  cudaError_t e = hfb::launchTilesPass(c, *u, *h, pos, tan, depth, strandsToRender, r);
  if (e != cudaSuccess) return fail(c, HFB_ERR_CUDA, std::string("tiles_pass_noalloc: ") + cudaGetErrorString(e));
  return HFB_OK;
}
