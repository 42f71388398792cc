/*
 * hairfb.h -- C-ABI of libhairfb.so, the GB300 (sm_103a) hair hot path.
 *
 * One entry point per WGSL compute pass of the reference renderer
 * (Scthe/frostbitten-hair-webgpu, src/passes/...), with the same inputs and
 * outputs as the pass's bind group and the same buffer byte layouts, so a
 * host that drove the WebGPU passes can drive these instead.  The reference's
 * per-pass interface is ``new XPass(device)`` + ``onViewportResize`` +
 * ``cmdClearBeforeRender`` + ``cmdX(ctx, hairObject)``
 * (e.g. src/passes/swHair/hairTilesPass.ts:22-140); here the pass constants
 * live in the context (HfbConfig), the viewport-sized buffers in
 * HfbRasterBuffers, and each ``cmdX`` is an ``hfb_*`` call.
 *
 * Conventions
 *   - Every function returns an int status: HFB_OK (0) or a negative
 *     HFB_ERR_* code; hfb_last_error() returns the message of the last failure
 *     on that context.  No C++ exception crosses this boundary.
 *   - Device buffers are plain CUDA device pointers (from hfb_buffer_alloc or
 *     any other CUDA allocator).  Host pointers are borrowed for the duration
 *     of the call only.  Uniform blocks are passed as host pointers to their
 *     raw bytes, as the reference uploads them with queue.writeBuffer.
 *   - Calls are asynchronous on the context's CUDA stream unless documented
 *     otherwise (like commands recorded into one WebGPU command encoder).
 *   - One context is used by one host thread at a time.
 */
#ifndef HAIRFB_H
#define HAIRFB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HFB_VERSION 1

#if defined(__GNUC__)
#define HFB_API __attribute__((visibility("default")))
#else
#define HFB_API
#endif

#define HFB_OK 0
#define HFB_ERR_INVALID_ARGUMENT (-1)
#define HFB_ERR_OUT_OF_MEMORY (-2)
#define HFB_ERR_CUDA (-3)
#define HFB_ERR_UNSUPPORTED (-6)

/* Pass constants the reference splices into its WGSL at pipeline creation
 * (CONFIG, src/constants.ts:86-349).  64 bytes. */
typedef struct HfbConfig {
  uint32_t tileSize;                        /* hairRender.tileSize: 8, 16 or 32 */
  uint32_t tileDepthBins;                   /* hairRender.tileDepthBins (<= 64) */
  uint32_t slicesPerPixel;                  /* hairRender.slicesPerPixel (<= 16; <= 8 with 32 px tiles) */
  uint32_t shadingPoints;                   /* hairRender.shadingPoints */
  uint32_t gridDims;                        /* hairSimulation.physicsForcesGrid.dims */
  uint32_t sortBuckets;                     /* hairRender.sortBuckets (<= 256) */
  uint32_t sortBucketSize;                  /* hairRender.sortBucketSize */
  uint32_t avgSegmentsPerTile;              /* hairRender.avgSegmentsPerTile */
  uint32_t avgFragmentsPerSlice;            /* hairRender.avgFragmentsPerSlice */
  uint32_t invalidTilesPerSegmentThreshold; /* hairRender.invalidTilesPerSegmentThreshold */
  uint32_t processorCount;                  /* fine-pass persistent CTAs; 0 = one wave */
  uint32_t alphaQuadratic;                  /* hairRender.alphaQuadratic (0/1) */
  float alphaMultiplier;                    /* hairRender.alphaMultipler */
  float cameraNear, cameraFar;              /* camera.projection (linearizeDepth) */
  uint32_t reserved;
} HfbConfig;

/* struct HairData, src/scene/hair/hairDataBuffer.ts:15-19 (padded). */
typedef struct HfbHairData {
  float boundingSphere[4]; /* xyz centre, w radius (object space) */
  uint32_t strandsCount;
  uint32_t pointsPerStrand; /* 2..256 */
  uint32_t padding[2];
} HfbHairData;

typedef struct HfbMat4 { float m[16]; } HfbMat4; /* column-major */
typedef struct HfbVec4 { float x, y, z, w; } HfbVec4;

/* struct Uniforms, src/passes/renderUniformsBuffer.ts:105-137 (1184 bytes). */
typedef struct HfbUniforms {
  HfbMat4 vpMatrix, vpMatrixInv, viewMatrix, projMatrix, projMatrixInv;
  HfbMat4 modelMatrix, modelViewMat, mvpMatrix, collisionSphereModelMatrix;
  HfbVec4 viewport;       /* width, height, 0, 0 */
  HfbVec4 cameraPosition; /* world space */
  HfbVec4 colorMgmt, lightAmbient;
  struct { HfbVec4 position, colorAndEnergy; } light0, light1, light2;
  struct {
    HfbMat4 sourceModelViewMat, sourceProjMatrix, sourceMVP_Matrix;
    HfbVec4 sourcePosition;
    uint32_t usePCSS, PCF_Radius;
    float bias, strength;
  } shadows;
  struct {
    float radius, directionOffset, falloffStart2, falloffEnd2;
    uint32_t numDirections, numSteps;
    float strength, padding0;
  } ao;
  struct {
    float color0[3]; float specular;
    float color1[3]; float shadows;
    float weightTT, weightTRT, shift, roughness;
    float colorRng, lumaRng, attenuation, padding1;
  } hairMaterial;
  struct { HfbVec4 boundsMin, boundsMax; } sdf;
  struct { HfbVec4 boundsMin; float boundsMax[3]; uint32_t debugDisplayValue; } gridData;
  float fiberRadius, dbgShadowMapPreviewSize;
  uint32_t maxDrawnHairSegments; /* 1 + tiles * avgSegmentsPerTile */
  uint32_t displayMode;          /* low 8 bits mode, bits 8..23 extra */
  float background[8];
  float collisionSpherePosition[3];
  uint32_t gizmoActiveState;
} HfbUniforms;

/* struct SimulationUniforms, src/passes/simulation/simulationUniformsBuffer.ts:19-51 (304 bytes). */
typedef struct HfbSimUniforms {
  HfbMat4 modelMatrix, modelMatrixInv;
  HfbVec4 collisionSphere; /* object space xyz, radius */
  HfbVec4 wind;            /* object-space direction xyz, strength */
  struct { HfbVec4 boundsMin, boundsMax; } sdf; /* boundsMax.w = distanceOffset */
  struct { HfbVec4 boundsMin; float boundsMax[3]; uint32_t debugDisplayValue; } gridData;
  float deltaTime, gravity;
  uint32_t constraintIterations, frameIdx;
  float windStrengthLull, windColisionTraceOffset, stiffnessLengthConstr, stiffnessCollisions;
  float stiffnessSDF, volumePreservation, friction, stiffnessGlobalConstr;
  float globalConstrExtent, globalConstrFade, stiffnessLocalConstr, windPhaseOffset;
  float windStrengthFrequency, windStrengthJitter, padding0, padding1;
} HfbSimUniforms;

/*
 * Viewport-sized buffers of the raster passes, in the reference layouts
 * (created by the passes' onViewportResize in the reference).  T = tile
 * count, B = tileDepthBins, maxDrawn = Uniforms.maxDrawnHairSegments.
 */
typedef struct HfbRasterBuffers {
  uint32_t width, height;
  uint32_t maxDrawnSegments;
  uint32_t reserved0;
  /* HairTileResult[T*B] {minDepth, maxDepth, tileSegmentPtr, pad}
   * (src/passes/swHair/shared/hairTilesResultBuffer.ts:77-82) */
  uint32_t* tiles;
  /* DrawnHairSegments {u32 drawnSegmentsCount; {strandAndSegmentIdxs, next}[maxDrawn]}
   * with the array at byte offset 4 (hairTileSegmentsBuffer.ts:60-68) */
  uint32_t* tileSegments;
  /* u32[T] (segmentCountPerTileBuffer.ts:10-45) */
  uint32_t* segmentCountPerTile;
  /* SortBucket[sortBuckets] {tileCount, writeOffset} (hairTileSortPass.countTiles.wgsl.ts:42-49) */
  uint32_t* sortBuckets;
  /* TilesList {u32 drawnTiles; u32 data[T]} (tileListBuffer.ts:15-19), 4 + T words */
  uint32_t* tileList;
  /* HairRasterResult {u32 tileQueueAtomicIdx; pad; vec4f data[W*H]} with the
   * array at byte offset 16 (hairRasterizerResultBuffer.ts:28-34).  Sized
   * 16 + 16*W*H bytes: one vec4f more than the reference, whose last pixel
   * falls outside its buffer. */
  float* rasterizerResult;
  /* working memory of the tiles pass, hfb_raster_scratch_bytes() bytes */
  void* scratch;
  size_t scratchBytes;
} HfbRasterBuffers;

/* Counters accumulated over the context's lifetime (read with hfb_get_counters).
 * No kernel of the library waits on another block, stream or rank (the
 * persistent kernels take work from atomic counters and a split tile's last
 * group merges it), so there is no device wait to time out or count. */
typedef struct HfbCounters {
  uint64_t tileRecords;        /* (segment, tile) records attempted (sum of drawnSegmentsCount) */
  uint64_t tileRecordsDropped; /* records lost because the segment pool was full */
  uint64_t finePoolFullBins;   /* tile depth bins whose fragment pool filled (fine pass break) */
  uint64_t launches;           /* kernels launched by the library */
  uint64_t fineSplitTiles;     /* fine pass: tiles split into groups of depth bins across CTAs */
  uint64_t fineSplitRedone;    /* fine pass: split tiles redone in order (a later group could fill a pool) */
  uint64_t badWorkItems;       /* fine-pass work items that failed their bounds checks (0 expected) */
} HfbCounters;

typedef struct HfbCtx HfbCtx;

/* ---- context ------------------------------------------------------------ */
HFB_API int hfb_version(void);
/* Validates the config (the WGSL constants) and binds the current CUDA
 * device `device` (-1 = keep current).  Creates the context's stream. */
HFB_API int hfb_ctx_create(const HfbConfig* cfg, int device, HfbCtx** out);
HFB_API int hfb_ctx_destroy(HfbCtx* ctx);
HFB_API const char* hfb_last_error(const HfbCtx* ctx);
/* Run subsequent calls on `stream` (a cudaStream_t, including the special
 * handles cudaStreamLegacy / cudaStreamPerThread); NULL restores the
 * context's own stream. */
HFB_API int hfb_ctx_set_stream(HfbCtx* ctx, void* stream);
/* Blocks until all work of the context's stream has finished. */
HFB_API int hfb_sync(HfbCtx* ctx);
/* Synchronizes, then copies the counters. */
HFB_API int hfb_get_counters(HfbCtx* ctx, HfbCounters* out);
/* Self-check of the simulation's divisions by the constants 3 and 1e6, which
 * its kernels compute as correctly rounded multiplications by the reciprocal
 * (one multiply and one FMA): compares them with the device's IEEE division
 * over all 2^32 inputs and writes the mismatch counts, all 0 expected:
 * out[0] x / 3 over every non-NaN float, out[1] (float)v / 1e6 over every
 * int32 v, out[2] x / 1e6 over every finite float with |x| >= 2^-92.
 * Synchronizes. */
HFB_API int hfb_check_constant_division(HfbCtx* ctx, uint64_t out[3]);

/* ---- buffers ------------------------------------------------------------ */
HFB_API int hfb_buffer_alloc(HfbCtx* ctx, size_t bytes, void** out);
HFB_API int hfb_buffer_free(HfbCtx* ctx, void* ptr);
HFB_API int hfb_buffer_upload(HfbCtx* ctx, void* dst, const void* src, size_t bytes);
/* Synchronous device -> host copy. */
HFB_API int hfb_buffer_download(HfbCtx* ctx, void* dst, const void* src, size_t bytes);
HFB_API int hfb_buffer_clear(HfbCtx* ctx, void* dst, size_t bytes);

/* Bytes of tiles-pass working memory for a viewport (segment pool sized by
 * the config: 1 + tiles * avgSegmentsPerTile), or for a given pool size. */
HFB_API size_t hfb_raster_scratch_bytes(const HfbConfig* cfg, uint32_t width, uint32_t height);
HFB_API size_t hfb_raster_scratch_bytes_for(const HfbConfig* cfg, uint32_t width, uint32_t height,
                                            uint32_t maxDrawnSegments);
/* onViewportResize of HairTilesPass / HairTileSortPass / HairFinePass:
 * allocates every HfbRasterBuffers member for width x height, with the
 * segment pool the reference sizes (getLengthOfHairTileSegmentsBuffer,
 * hairTileSegmentsBuffer.ts:81-87). */
HFB_API int hfb_raster_buffers_alloc(HfbCtx* ctx, uint32_t width, uint32_t height, HfbRasterBuffers* out);
/* No counterpart in the reference: the same with a segment pool of
 * maxDrawnSegments records, for hosts that size each instance's pool (a
 * server mixing dense small viewports with sparse large ones).  The frame's
 * Uniforms.maxDrawnHairSegments must carry the same number. */
HFB_API int hfb_raster_buffers_alloc_sized(HfbCtx* ctx, uint32_t width, uint32_t height, uint32_t maxDrawnSegments,
                                           HfbRasterBuffers* out);
HFB_API int hfb_raster_buffers_free(HfbCtx* ctx, HfbRasterBuffers* rb);

/* ---- simulation passes (src/renderer.ts:212-240 order) --------------------- */

/* GridPreSimPass.cmdUpdateGridsBeforeSim (gridPreSimPass.ts:34-62,
 * gridPreSimPass.wgsl.ts:38-159): densityGradWind[G^3] {vec3f grad, f32 wind}
 * from the previous frame's densityVelocity[G^3] {i32 vx, vy, vz, density}
 * and the SDF (sdfDims^3 f32, x fastest). */
HFB_API int hfb_grid_pre_sim(HfbCtx* ctx, const HfbSimUniforms* u, const int32_t* densityVelocity,
                     float* densityGradWind, const float* sdf, uint32_t sdfDims);

/* HairSimIntegrationPass.cmdSimulateHairPositions (hairSimIntegrationPass.ts:33-60,
 * hairSimIntegrationPass.wgsl.ts:79-273): reads positionsPrev and positionsNow
 * (vec4f, .w = isMovable), writes the new positions into positionsPrev.  The
 * caller then swaps its "current" buffer (HairObject.swapPositionBuffersAfterSimIntegration). */
HFB_API int hfb_sim_integrate(HfbCtx* ctx, const HfbSimUniforms* u, const HfbHairData* hair,
                      float* positionsPrev, const float* positionsNow, const float* positionsInitial,
                      const float* segmentLengths, const int32_t* densityVelocity,
                      const float* densityGradWind, const float* sdf, uint32_t sdfDims);

/* GridPostSimPass.cmdUpdateGridsAfterSim (gridPostSimPass.ts:33-59,
 * gridPostSimPass.wgsl.ts:45-72): clears densityVelocity, then splats
 * velocity (now - prev) and density of every point into it. */
HFB_API int hfb_grid_post_sim(HfbCtx* ctx, const HfbSimUniforms* u, const HfbHairData* hair,
                      const float* positionsPrev, const float* positionsNow, int32_t* densityVelocity);

/* hfb_grid_post_sim visiting the strands in the order strandOrder (device,
 * strandsCount u32, a permutation; NULL = 0, 1, 2, ...).  The splat is a sum
 * of wrapping i32 adds, so the grid is the same for every order; an order
 * that puts neighbouring strands next to each other (hfb_strand_grid_order)
 * lets a block merge more of its adds before they reach global memory. */
HFB_API int hfb_grid_post_sim_ordered(HfbCtx* ctx, const HfbSimUniforms* u, const HfbHairData* hair,
                              const float* positionsPrev, const float* positionsNow, int32_t* densityVelocity,
                              const uint32_t* strandOrder);

/* Host: the strands of a hair asset (positions: host, strandsCount *
 * pointsPerStrand vec4f) sorted by the Morton code of their root within the
 * roots' bounding box (10 bits per axis; ties keep strand order).  Writes
 * strandsCount indices to orderOut (host). */
HFB_API int hfb_strand_grid_order(const float* positions, uint32_t strandsCount, uint32_t pointsPerStrand,
                          uint32_t* orderOut);

/* ---- shading (HairShadingPass.cmdComputeShadingPoints, hairShadingPass.ts:41-68) ---- */
/* depth: width*height f32 (row 0 = top); ao: aoWidth*aoHeight f32 or NULL
 * (unoccluded); shadowMap: shadowMapSize^2 f32 or NULL (no shadow).
 * shading: strandsCount*shadingPoints vec4f. */
HFB_API int hfb_shading(HfbCtx* ctx, const HfbUniforms* u, const HfbHairData* hair, const float* positions,
                const float* tangents, const float* depth, const float* ao, uint32_t aoWidth,
                uint32_t aoHeight, const float* shadowMap, uint32_t shadowMapSize, float* shading);

/* ---- software raster (src/renderer.ts:263-277 order) ---------------------- */

/* cmdClearBeforeRender of HairTilesPass, HairFinePass and HairTileSortPass
 * (hairTilesPass.ts:48-52, hairFinePass.ts:50-55, hairTileSortPass.ts:63-68). */
HFB_API int hfb_clear_before_render(HfbCtx* ctx, HfbRasterBuffers* rb);

/* HairTilesPass.cmdDrawHairToTiles (hairTilesPass.wgsl.ts:70-246): bins the
 * segments of the first strandsToRender strands into per-tile depth-bin
 * lists.  depth: the scene depth buffer, width*height f32, row 0 = top.
 * The lists come out in a canonical order: within each (tile, depth bin)
 * the list walks segments in descending (strand, segment) order. */
HFB_API int hfb_tiles_pass(HfbCtx* ctx, const HfbUniforms* u, const HfbHairData* hair, const float* positions,
                   const float* tangents, const float* depth, uint32_t strandsToRender,
                   HfbRasterBuffers* rb);

/* HairTileSortPass.cmdSortHairTiles (count-tiles + sort kernels): tile list,
 * heaviest bucket first; within a bucket, ascending tile index. */
HFB_API int hfb_tile_sort(HfbCtx* ctx, HfbRasterBuffers* rb);

/* HairFinePass.cmdRasterizeSlicesHair (hairFinePass.wgsl.ts:126-335):
 * persistent CTAs take tiles from the queue, blend every depth bin's
 * segments front to back into rasterizerResult. shading: the strand-space
 * colours (S*shadingPoints vec4f). */
HFB_API int hfb_fine_pass(HfbCtx* ctx, const HfbUniforms* u, const HfbHairData* hair, const float* positions,
                  const float* tangents, const float* shading, const float* depth,
                  HfbRasterBuffers* rb);

/* ---- whole frames (src/renderer.ts:171-295 order) -------------------------- */

/* One hair instance of a frame: its resident buffers and this frame's
 * uniforms.  A frame runs, in the reference's order, GridPreSimPass,
 * HairSimIntegrationPass (then the position swap), GridPostSimPass, the
 * raster clears, HairTilesPass, HairTileSortPass, HairFinePass and
 * HairShadingPass (whose result the next frame samples). */
typedef struct HfbInstance {
  const HfbUniforms* uniforms;        /* host, read during the call */
  const HfbSimUniforms* simUniforms;  /* host, read during the call */
  HfbHairData hair;
  /* tick-tock positions (vec4f, .w = isMovable): positions[current] is
   * "now", the other "prev" (hairPointsPositionsBuffer.ts).  Integration
   * writes the new positions over "prev" and the frame flips `current`
   * (HairObject.swapPositionBuffersAfterSimIntegration). */
  float* positions[2];
  uint32_t current;
  uint32_t strandsToRender;           /* LOD: strands drawn by the tiles pass */
  const float* positionsInitial;
  const float* tangents;
  const float* segmentLengths;
  int32_t* densityVelocity;           /* G^3 {i32 vx, vy, vz, density} */
  float* densityGradWind;             /* G^3 {vec3f grad, f32 wind} */
  const float* sdf;
  uint32_t sdfDims;
  uint32_t shadowMapSize;
  float* shading;                     /* S*SP vec4f */
  const float* sceneDepth;            /* W*H f32: tiles / fine depth tests */
  const float* shadingDepth;          /* W*H f32: shading attenuation; NULL = sceneDepth */
  const float* ao;                    /* NULL = unoccluded */
  uint32_t aoWidth, aoHeight;
  const float* shadowMap;             /* NULL = unshadowed */
  HfbRasterBuffers raster;            /* from hfb_raster_buffers_alloc */
  /* W*H f32, NULL = none.  If set, the frame copies sceneDepth into it and
   * draws the hair's depth over it after the fine pass (hfb_hair_depth), and
   * the shading pass reads it instead of shadingDepth: the depth buffer with
   * the hair drawn that HwHairPass leaves for the shading
   * (renderer.ts:286-296). */
  float* hairDepth;
  /* device, strandsCount u32 or NULL: the order the grid splat visits the
   * strands in (hfb_grid_post_sim_ordered) */
  const uint32_t* gridOrder;
} HfbInstance;

/* HwHairPass.cmdDrawHair's depth output (hwHairPass.ts:71-160): copies
 * sceneDepth (W*H f32) into hairDepth and draws every rendered hair segment's
 * two triangles (hwRasterizeHair.wgsl.ts:23-57) over it with depth test
 * 'less'.  Coverage at pixel centres, edges inclusive, depth = NDC z
 * interpolated in screen space; the GPU rasterizer's own snapping and
 * depth24 storage are not reproduced.  Uses rb's scratch as working memory
 * (the raster passes' scratch is free after the fine pass). */
/* HairCombinePass + PresentPass (hairCombinePass.wgsl.ts:51-89 with its
 * src-alpha blend, presentPass.wgsl.ts main_fs in DISPLAY_MODE_FINAL): the
 * fine pass's result (rb, read upside down as the combine pass does) over
 * sceneColor (W*H vec4f, row 0 at the top; NULL = black), then the 8x8
 * Bayer dither, exposure, ACES tone mapping and gamma of Uniforms.colorMgmt
 * (gamma, exposure, dither strength), stored as unorm8: rgba is W*H RGBA8
 * (device), row 0 at the top, alpha 255. */
HFB_API int hfb_present(HfbCtx* ctx, const HfbUniforms* uniforms, const HfbRasterBuffers* rb,
                        const float* sceneColor, uint8_t* rgba);

/* hfb_present for the images of many instances (those of a batched frame),
 * in one launch per 64 images: items[k] holds one hfb_present call's
 * arguments, each checked as hfb_present checks them before any launch, and
 * each image equals what hfb_present makes of the same arguments. */
typedef struct HfbPresentItem {
  const HfbUniforms* uniforms;
  const HfbRasterBuffers* rb;
  const float* sceneColor; /* NULL = black */
  uint8_t* rgba;
} HfbPresentItem;
HFB_API int hfb_present_batch(HfbCtx* ctx, const HfbPresentItem* items, uint32_t n);

/* HwHairPass.cmdDrawHair's normal output (hwHairPass.wgsl.ts:88-97): at every
 * pixel where the hair is in front (its depth equals hairDepth, as
 * hfb_hair_depth left it), the octahedron encoding of the normalised
 * tangent the fragment interpolates (perspective-correct) from
 * modelMatrix * (tangent, 1), stored as rg16float values; the fragment
 * that wins a pixel is the first drawn among those at its depth (strand,
 * segment, triangle order).  normals: W*H vec2f (device), in/out: pixels
 * without hair keep their value (the scene's normals, or 0 as the
 * reference clears them).  winner: W*H u32 of device working memory. */
HFB_API int hfb_hair_normals(HfbCtx* ctx, const HfbUniforms* uniforms, const HfbHairData* hair,
                             const float* positions, const float* tangents, uint32_t strandsToRender,
                             const float* hairDepth, float* normals, uint32_t* winner, HfbRasterBuffers* rb);

/* AoPass.cmdCalcAo (aoPass.wgsl.ts, gtao.wgsl.ts): ground-truth ambient
 * occlusion at ceil(W*scale) x ceil(H*scale) texels (the reference's
 * CONFIG.ao.textureSizeMul, 0.5) from depth (W*H f32, e.g. hfb_hair_depth's)
 * and normals (W*H vec2f octahedron, e.g. hfb_hair_normals'), with the
 * Uniforms.ao parameters; stored as r16float values in ao (device f32).
 * The shading reads it (hfb_shading's ao, aoWidth, aoHeight). */
HFB_API int hfb_gtao(HfbCtx* ctx, const HfbUniforms* uniforms, const float* depth, const float* normals, float scale,
                     float* ao);

HFB_API int hfb_hair_depth(HfbCtx* ctx, const HfbUniforms* uniforms, const HfbHairData* hair, const float* positions,
                           const float* tangents, uint32_t strandsToRender, const float* sceneDepth,
                           float* hairDepth, HfbRasterBuffers* rb);

/* One frame of one instance (the per-pass entries above, in order). */
HFB_API int hfb_frame(HfbCtx* ctx, HfbInstance* instance);

/* No single counterpart in the reference, which renders one hair object per
 * frame.  One frame of n instances of uneven strand counts, points per
 * strand and viewports: every pass runs as one persistent launch over all
 * instances (instance-offset tables in device memory), the launch sequence
 * is a CUDA graph captured once per context, and the fine pass pulls the
 * tiles of all instances from one queue.  The context's config (tile size,
 * depth bins, slices, grid size) applies to every instance.  Results are
 * those of hfb_frame on each instance alone.  The call flips every
 * instance's `current`.  n <= 1024. */
HFB_API int hfb_frame_batch(HfbCtx* ctx, HfbInstance* instances, uint32_t n);

/* No counterpart in the reference.  Splits the instances of the following
 * hfb_frame_batch calls into `groups` (1..4, default 1) groups of about equal
 * work, each running its passes on its own stream with 1/groups of the GPU's
 * persistent CTAs, so that different passes of different groups share the
 * SMs.  Results do not depend on it. */
HFB_API int hfb_ctx_set_batch_groups(HfbCtx* ctx, uint32_t groups);

/* No counterpart in the reference.  With on = 1, hfb_frame_batch runs the
 * simulation passes and the raster passes of a frame on two internal streams
 * with two device tables in turn, so that a frame's simulation runs beside
 * the previous frame's raster passes (one group; groups are ignored).  A
 * frame's results are ordered on the context's stream as before, but its
 * simulation does not wait for work the caller enqueued on that stream after
 * the previous hfb_frame_batch call: inputs such a frame reads (the instances'
 * device buffers) must be ready when the call is made.  Switching waits for
 * the device. */
HFB_API int hfb_ctx_set_batch_pipeline(HfbCtx* ctx, uint32_t on);

/* hfb_frame_batch run as plain launches with a CUDA event between passes;
 * waits for the frame and writes the GPU time of each pass, in ms, to
 * passMs[0..8]: grid_pre, integrate, grid_post (with its grid clear),
 * clear (the raster clears), tiles, sort, fine, hair_depth, shading.  For
 * profiling. */
#define HFB_FRAME_PASSES 9
HFB_API int hfb_frame_batch_profile(HfbCtx* ctx, HfbInstance* instances, uint32_t n, float* passMs);

/* No counterpart in the reference.  hfb_tiles_pass for callers that cannot
 * allocate device memory (a render thread that must not take cudaMalloc's
 * device-wide synchronisation, a host whose allocator owns every device
 * byte, code about to record a stream capture).  Same inputs, outputs and
 * results as hfb_tiles_pass, but the pass's working memory comes from one
 * fixed array of HFB_NOALLOC_SCRATCH_BYTES compiled into the library, held
 * by every GPU that loads it until exit; rb->scratch is ignored and may be
 * NULL.  Viewports needing more (hfb_raster_scratch_bytes) are rejected with
 * HFB_ERR_INVALID_ARGUMENT.  Calls share the array: calls whose work
 * overlaps on the GPU race.  hfb_ctx_create looks the array's address up
 * (cudaGetSymbolAddress, with the context's device current) and loads the
 * pass's kernels, which is when the array and the code take their device
 * memory (CUDA loads device code lazily); the call itself allocates
 * nothing. */
#define HFB_NOALLOC_SCRATCH_BYTES (16u << 20)
HFB_API int hfb_tiles_pass_noalloc(HfbCtx* ctx, const HfbUniforms* u, const HfbHairData* hair,
                                   const float* positions, const float* tangents, const float* depth,
                                   uint32_t strandsToRender, HfbRasterBuffers* rb);

#ifdef __cplusplus
} /* extern "C" */
#endif

#ifdef __cplusplus
static_assert(sizeof(HfbConfig) == 64, "HfbConfig layout");
static_assert(sizeof(HfbHairData) == 32, "HfbHairData layout");
static_assert(sizeof(HfbUniforms) == 1184, "Uniforms layout");
static_assert(sizeof(HfbSimUniforms) == 304, "SimulationUniforms layout");
static_assert(sizeof(HfbInstance) == 272, "HfbInstance layout");
static_assert(sizeof(HfbPresentItem) == 32, "HfbPresentItem layout");
#else
_Static_assert(sizeof(HfbConfig) == 64, "HfbConfig layout");
_Static_assert(sizeof(HfbHairData) == 32, "HfbHairData layout");
_Static_assert(sizeof(HfbUniforms) == 1184, "Uniforms layout");
_Static_assert(sizeof(HfbSimUniforms) == 304, "SimulationUniforms layout");
_Static_assert(sizeof(HfbInstance) == 272, "HfbInstance layout");
_Static_assert(sizeof(HfbPresentItem) == 32, "HfbPresentItem layout");
#endif

#endif /* HAIRFB_H */
