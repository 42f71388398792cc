// Hair depth prepass: HwHairPass.cmdDrawHair's depth output as CUDA.
//
// The reference draws every hair segment as two triangles with the hardware
// rasterizer (hwHairPass.ts:71-160, vertex shader hwRasterizeHair,
// hwRasterizeHair.wgsl.ts:23-57, index order hairIndexBuffer.ts:29-46) into
// the depth buffer that already holds the scene, with depthCompare 'less'
// (PIPELINE_DEPTH_ON, passes/_shared/shared.ts:22-26).  The shading pass then
// reads that depth (renderer.ts:286-296).  This restates it:
//
// - vertex 2*id + k of segment id = strand*P + seg (k = 0..3) is point
//   seg + k/2 in view space (modelViewMat), moved by fiberRadius along
//   safeNormalize(cross(tangentVS, (0, 0, 1))) -- plus for even k, minus for
//   odd k (the tangent is transformed with w = 1, as the reference does) --
//   and projected (projMatrix); triangles (0, 1, 2) and (2, 1, 3);
// - coverage is tested at pixel centres (x + 0.5, y + 0.5) in framebuffer
//   coordinates (rows down), both windings drawn (cullMode 'none'), edges
//   inclusive; depth = NDC z interpolated with the screen-space barycentric
//   weights, as (w0 z0 + w1 z1 + w2 z2) / area (the edge values w_i summed
//   before the one division); a triangle with a vertex behind the camera (w <= 0) is not
//   drawn (no near-plane clipping); depth outside [0, 1] is discarded;
// - the 'less' test is an atomic minimum on the depth's bits (non-negative
//   floats order like their bits), so the result does not depend on the
//   order of the fragments.
// The GPU's own rasterizer rules (fixed-point vertex snapping, the top-left
// tie-break, depth24 storage) are implementation-defined and not reproduced;
// the oracle (oracle_hair_depth) follows the rules above.
#define HFB_TU 7
#include <cuda_fp16.h>

#include "hfb_internal.cuh"
#include "hfb_math.cuh"

namespace hfb {
namespace {

constexpr uint32_t HD_THREADS = 256;             // points per block: each point's two vertices once
constexpr uint32_t HD_WARP_SEGS = 31;            // segment starts per warp: its 32 points, the last shared
constexpr uint32_t HD_SEGS = (HD_THREADS / 32u) * HD_WARP_SEGS;  // segment starts per block
constexpr uint32_t HD_BIG_AREA = 1024;           // pixels: larger triangles are drawn by a whole block
constexpr uint32_t HD_VIEW_FLOATS = 35;

// The uniforms the pass reads: modelViewMat, projMatrix, fiberRadius, viewport.
struct HdView {
  float mv[16], pr[16];
  float radius, W, H;
};
static_assert(sizeof(HdView) == HD_VIEW_FLOATS * 4, "HdView layout");

__host__ __device__ inline float hdViewField(const HfbUniforms& U, uint32_t k) {
  return k < 16u ? U.modelViewMat.m[k] : k < 32u ? U.projMatrix.m[k - 16u]
                                        : k == 32u ? U.fiberRadius : k == 33u ? U.viewport.x : U.viewport.y;
}

inline HdView hdView(const HfbUniforms& U) {
  HdView v;
  float* f = reinterpret_cast<float*>(&v);
  for (uint32_t k = 0; k < HD_VIEW_FLOATS; k++) f[k] = hdViewField(U, k);
  return v;
}

struct ScreenV {
  float x, y, z;
  bool ok;
};

struct Tri {
  ScreenV v[3];
};

__device__ __forceinline__ float edgeFn(float ax, float ay, float bx, float by, float px, float py) {
  return fsub(fmul(fsub(bx, ax), fsub(py, ay)), fmul(fsub(by, ay), fsub(px, ax)));
}

__device__ __forceinline__ ScreenV projectScreen(const HdView& V, f3 e) {
  const f4 clip = m4v(V.pr, mk4(e.x, e.y, e.z, 1.0f));
  ScreenV v;
  v.ok = clip.w > 0.0f;
  const float nx = clip.x / clip.w, ny = clip.y / clip.w;
  v.z = clip.z / clip.w;
  v.x = fmul(fadd(fmul(nx, 0.5f), 0.5f), V.W);
  v.y = fmul(fsub(0.5f, fmul(ny, 0.5f)), V.H);
  return v;
}

// The two vertices of point i: in view space (modelViewMat), moved by
// fiberRadius along safeNormalize(cross(tangentVS, (0, 0, 1))) -- plus for
// `a` (even vertex ids), minus for `b` (odd ones) -- and projected.
__device__ __forceinline__ void pointPair(const HdView& V, const float4* __restrict__ pos,
                                          const float4* __restrict__ tan, size_t i, ScreenV& a, ScreenV& b) {
  const float4 p = __ldg(HFB_G(&pos[i]));
  const float4 t = __ldg(HFB_G(&tan[i]));
  const f4 pVS = m4v(V.mv, mk4(p.x, p.y, p.z, 1.0f));
  const f4 tVS = m4v(V.mv, mk4(t.x, t.y, t.z, 1.0f));
  const f3 c = cross3(xyz(tVS), mk3(0.0f, 0.0f, 1.0f));
  const f3 right = dot3(c, c) >= 1e-7f ? norm3(c) : mk3(0.0f, 0.0f, 0.0f);  // safeNormalize3
  const f3 th = mul3s(right, V.radius);
  a = projectScreen(V, add3(xyz(pVS), th));
  b = projectScreen(V, sub3(xyz(pVS), th));
}

__device__ __forceinline__ float4 packV(const ScreenV& v) { return make_float4(v.x, v.y, v.z, v.ok ? 1.0f : 0.0f); }
__device__ __forceinline__ ScreenV unpackV(float4 f) { return {f.x, f.y, f.z, f.w != 0.0f}; }

// Pixel range [x0, x1] x [y0, y1] whose centres lie in the triangle's box;
// false if the triangle is not drawn at all.
__device__ __forceinline__ bool triBox(const Tri& t, uint32_t W, uint32_t H, float& area, int& x0, int& x1, int& y0,
                                       int& y1) {
  if (!t.v[0].ok || !t.v[1].ok || !t.v[2].ok) return false;
  area = edgeFn(t.v[0].x, t.v[0].y, t.v[1].x, t.v[1].y, t.v[2].x, t.v[2].y);
  if (!(area != 0.0f) || !isfinite(area)) return false;
  const float mnx = fminf(fminf(t.v[0].x, t.v[1].x), t.v[2].x), mxx = fmaxf(fmaxf(t.v[0].x, t.v[1].x), t.v[2].x);
  const float mny = fminf(fminf(t.v[0].y, t.v[1].y), t.v[2].y), mxy = fmaxf(fmaxf(t.v[0].y, t.v[1].y), t.v[2].y);
  if (!(mxx >= 0.5f && mxy >= 0.5f && mnx <= (float)W - 0.5f && mny <= (float)H - 0.5f)) return false;
  x0 = (int)fmaxf(ceilf(fsub(mnx, 0.5f)), 0.0f);
  y0 = (int)fmaxf(ceilf(fsub(mny, 0.5f)), 0.0f);
  x1 = (int)fminf(floorf(fsub(mxx, 0.5f)), (float)W - 1.0f);
  y1 = (int)fminf(floorf(fsub(mxy, 0.5f)), (float)H - 1.0f);
  return x0 <= x1 && y0 <= y1;
}

// Where a pass writes: the depth ('less' test as an atomic minimum of the
// depth bits) or, in the winner pass (WIN), the smallest primitive index
// among the fragments whose depth equals the final one (the first drawn of
// equal depths keeps the pixel, as in draw order).
struct HdOut {
  unsigned* depth;
  unsigned* winner;
  uint32_t W;
};

template <bool WIN>
__device__ __forceinline__ void triPixel(const Tri& t, float area, const HdOut& o, int x, int y, uint32_t prim) {
  const float px = fadd((float)x, 0.5f), py = fadd((float)y, 0.5f);
  float w0 = edgeFn(t.v[1].x, t.v[1].y, t.v[2].x, t.v[2].y, px, py);
  float w1 = edgeFn(t.v[2].x, t.v[2].y, t.v[0].x, t.v[0].y, px, py);
  float w2 = edgeFn(t.v[0].x, t.v[0].y, t.v[1].x, t.v[1].y, px, py);
  if (area < 0.0f) { w0 = -w0; w1 = -w1; w2 = -w2; }
  if (!(w0 >= 0.0f && w1 >= 0.0f && w2 >= 0.0f)) return;
  const float a = fabsf(area);
  const float z = fadd(fadd(fmul(w0, t.v[0].z), fmul(w1, t.v[1].z)), fmul(w2, t.v[2].z)) / a;
  if (!(z >= 0.0f && z <= 1.0f)) return;
  const size_t p = (size_t)y * o.W + x;
  const unsigned zb = __float_as_uint(fadd(z, 0.0f));  // -0 -> +0
  if (WIN) {
    if (zb == *HFB_G(&o.depth[p])) atomicMin(HFB_G(&o.winner[p]), prim);
  } else {
    atomicMin(HFB_G(&o.depth[p]), zb);
  }
}

// Row y's pixels of the triangle: [L, R] (in: the box's x range) narrowed to
// the pixels whose centres pass all three edge tests of triPixel; false if
// none do.  For a fixed row an edge value fsub(C, fmul(B, fsub(px, ax)))
// is monotone in px (each rounded step is), so each edge passes on a prefix
// or a suffix of the row.  Its end is searched with the same float test,
// from the pixel where the edge crosses the row in real arithmetic:
// galloping away from that guess, then bisecting, so the span holds exactly
// the pixels the per-pixel test accepts whatever the guess.  Needs no
// overflow to infinity in the products (spanSafe).
__device__ __forceinline__ bool rowSpan(const Tri& t, bool neg, int y, int& L, int& R) {
  const float py = fadd((float)y, 0.5f);
#pragma unroll
  for (int e = 0; e < 3; e++) {
    // the edges of triPixel: w0 = (v1, v2), w1 = (v2, v0), w2 = (v0, v1)
    const ScreenV& a = t.v[e == 0 ? 1 : e == 1 ? 2 : 0];
    const ScreenV& b = t.v[e == 0 ? 2 : e == 1 ? 0 : 1];
    auto pass = [&](int x) {
      const float w = edgeFn(a.x, a.y, b.x, b.y, fadd((float)x, 0.5f), py);
      return (neg ? -w : w) >= 0.0f;
    };
    const float B = fsub(b.y, a.y);
    const float dir = neg ? -B : B;
    if (dir == 0.0f) {  // the edge value is the same along the row
      if (!pass(L)) return false;
      continue;
    }
    // the edge passes on a prefix of the row when dir > 0, on a suffix when
    // dir < 0; f is false then true along [L, R] either way, and the edge's
    // end is where f first holds (R + 1: never)
    const bool prefix = dir > 0.0f;
    auto f = [&](int x) { return prefix ? !pass(x) : pass(x); };
    const float cross = a.x + (py - a.y) * (b.x - a.x) / B - 0.5f;  // real-arithmetic guess
    const int g = (int)fminf(fmaxf(cross, (float)L), (float)R);
    int lo, hi;  // f(lo) false or lo = L - 1; f(hi) true or hi = R + 1
    if (f(g)) {
      hi = g;
      int step = 1;
      lo = g - 1;
      while (lo >= L && f(lo)) {
        hi = lo;
        lo = hi - (step <<= 1);
      }
      if (lo < L - 1) lo = L - 1;
    } else {
      lo = g;
      int step = 1;
      hi = g + 1;
      while (hi <= R && !f(hi)) {
        lo = hi;
        hi = lo + (step <<= 1);
      }
      if (hi > R + 1) hi = R + 1;
    }
    while (hi - lo > 1) {  // f(lo) false (or lo = L - 1), f(hi) true (or hi = R + 1)
      const int mid = lo + (hi - lo) / 2;
      if (f(mid)) hi = mid; else lo = mid;
    }
    // hi: the first x where f is true
    if (prefix) R = hi - 1; else L = hi;
    if (L > R) return false;
  }
  return true;
}

// Vertex coordinates below 1e18 in magnitude (pixel centres are far below):
// every difference stays below 2^61 and every product below 2^122, so the
// edge values are finite (no inf - inf) and rowSpan's monotonicity holds.
__device__ __forceinline__ bool spanSafe(const Tri& t) {
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 3; k++) ok = ok && fabsf(t.v[k].x) < 1e18f && fabsf(t.v[k].y) < 1e18f;
  return ok;
}

// Every pixel of the triangle's box [x0, x1] x [y0, y1], rows y0 + first,
// y0 + first + step, ...: by row spans, or pixel by pixel when spanSafe fails.
template <bool WIN>
__device__ __forceinline__ void drawRows(const Tri& t, float area, const HdOut& o, int x0, int x1, int y0, int y1,
                                         int first, int step, uint32_t prim) {
  const bool safe = spanSafe(t), neg = area < 0.0f;
  for (int y = y0 + first; y <= y1; y += step) {
    int L = x0, R = x1;
    if (safe && !rowSpan(t, neg, y, L, R)) continue;
    for (int x = L; x <= R; x++) triPixel<WIN>(t, area, o, x, y, prim);
  }
}

// Triangle tr of the segment whose quad is q: (0, 1, 2) or (2, 1, 3).
__device__ __forceinline__ Tri segTri(const ScreenV (&q)[4], uint32_t tr) {
  Tri t;
  t.v[0] = tr ? q[2] : q[0];
  t.v[1] = q[1];
  t.v[2] = tr ? q[3] : q[2];
  return t;
}

// A segment's two triangles for the warp's shared pixel loop: their pixel
// boxes (an empty box for a triangle not drawn here), areas, and the union
// of the boxes that the loop walks.
struct HdUnit {
  int bx0[2], bx1[2], by0[2], by1[2];
  float area[2];
  int x0, y0;
  uint32_t bw, divBw;  // union box width and ceil(2^32 / width) (0 for width 1: 2^32 does not fit)
};

struct HdShared {
  float4 sv[HD_THREADS][2];            // each point's two screen vertices (x, y, z, drawable)
  HdUnit unit[HD_THREADS];             // each thread's segment
  uint32_t start[HD_THREADS / 32][32]; // per warp: first pixel of each lane's union box
};

// The quad of the segment whose first point has block index k.
__device__ __forceinline__ void blockQuad(const HdShared& sh, uint32_t k, ScreenV (&q)[4]) {
  q[0] = unpackV(sh.sv[k][0]);
  q[1] = unpackV(sh.sv[k][1]);
  q[2] = unpackV(sh.sv[k + 1][0]);
  q[3] = unpackV(sh.sv[k + 1][1]);
}

// One block of segment starts [blk * HD_SEGS, (blk + 1) * HD_SEGS): each
// warp projects the two vertices of 32 consecutive points into shared
// memory and its first 31 lanes own the segments from their point to the
// next (when that point is not its strand's last): the warps need no
// barrier between them.  A lane boxes its segment's two triangles.  A box
// of more than HD_BIG_AREA pixels goes onto the big list (entries
// point << 1 | triangle; capacity `bigCap`); the pixels of the union of a
// segment's other boxes are shared out over the warp's lanes (an exclusive
// scan of the union sizes), each pixel tested against both triangles
// within their own boxes, so a lane with a long thin segment does not hold
// up the other 31.  A big triangle that finds the list full is drawn by its
// own thread.  Called by every thread of the block.
// prim: the primitive index of triangle tr of the segment from point pt,
// (strand * (P - 1) + segment) * 2 + tr, the order the reference draws them.
__device__ __forceinline__ uint32_t primOf(uint32_t pt, uint32_t P, uint32_t tr) {
  return ((pt - pt / P) << 1) | tr;
}

template <bool WIN>
__device__ __forceinline__ void hairDepthBlock(const HdView& V, uint32_t P, uint32_t nPts,
                                               const float4* __restrict__ pos, const float4* __restrict__ tan,
                                               const HdOut& out, uint32_t* __restrict__ big,
                                               uint32_t bigCap, uint32_t blk, HdShared& sh) {
  const uint32_t tid = threadIdx.x, lane = tid & 31u, wp = tid >> 5;
  // warp wp: points blk * HD_SEGS + wp * 31 + lane; its segments start at lanes 0..30,
  // so a segment's two points are projected by the same warp
  const uint32_t pt = blk * HD_SEGS + wp * HD_WARP_SEGS + lane;
  if (pt < nPts) {
    ScreenV a, b;
    pointPair(V, pos, tan, pt, a, b);
    sh.sv[tid][0] = packV(a);
    sh.sv[tid][1] = packV(b);
  }
  __syncwarp();
  const uint32_t W = f2u(V.W), H = f2u(V.H);
  uint32_t mine = 0;
  bool own[2] = {false, false};  // big, list full: drawn by this thread
  if (lane < HD_WARP_SEGS && pt + 1u < nPts && pt % P != P - 1u) {
    ScreenV q[4];
    blockQuad(sh, tid, q);
    HdUnit un;
    int ux0 = 0x7fffffff, uy0 = 0x7fffffff, ux1 = -1, uy1 = -1;
#pragma unroll
    for (uint32_t tr = 0; tr < 2u; tr++) {
      un.bx0[tr] = 1; un.bx1[tr] = 0; un.by0[tr] = 1; un.by1[tr] = 0;  // empty
      un.area[tr] = 0.0f;
      const Tri t = segTri(q, tr);
      float area;
      int x0, x1, y0, y1;
      if (!triBox(t, W, H, area, x0, x1, y0, y1)) continue;
      const uint32_t bw = (uint32_t)(x1 - x0 + 1), bh = (uint32_t)(y1 - y0 + 1);
      if ((uint64_t)bw * bh > HD_BIG_AREA) {
        const uint32_t slot = bigCap > 0u && pt < 0x80000000u ? atomicAdd(HFB_G(&big[0]), 1u) : bigCap;
        if (slot < bigCap)
          *HFB_G(&big[1u + slot]) = (pt << 1) | tr;
        else
          own[tr] = true;
        continue;
      }
      un.bx0[tr] = x0; un.bx1[tr] = x1; un.by0[tr] = y0; un.by1[tr] = y1;
      un.area[tr] = area;
      ux0 = min(ux0, x0); ux1 = max(ux1, x1); uy0 = min(uy0, y0); uy1 = max(uy1, y1);
    }
    if (ux1 >= ux0) {  // the union of the boxes drawn here
      un.x0 = ux0;
      un.y0 = uy0;
      un.bw = (uint32_t)(ux1 - ux0 + 1);
      un.divBw = un.bw > 1u ? (uint32_t)((0x100000000ull + un.bw - 1u) / un.bw) : 0u;
      mine = un.bw * (uint32_t)(uy1 - uy0 + 1);
      sh.unit[tid] = un;
    }
  }
  // exclusive scan of the lanes' union boxes
  uint32_t incl = mine;
#pragma unroll
  for (uint32_t d = 1; d < 32u; d <<= 1) {
    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  sh.start[wp][lane] = incl - mine;
  __syncwarp();
  for (uint32_t k = lane; k < total; k += 32u) {
    uint32_t lo = 0, hi = 31;  // the last lane whose pixels start at or before k owns pixel k
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1u) >> 1;
      if (sh.start[wp][mid] <= k) lo = mid; else hi = mid - 1u;
    }
    const uint32_t o = wp * 32u + lo;
    const HdUnit& un = sh.unit[o];
    const uint32_t local = k - sh.start[wp][lo];
    // the union of two boxes of at most HD_BIG_AREA pixels each is at most
    // 2048 wide and holds fewer than 2^21 pixels, so local * (divBw * bw - 2^32)
    // < 2^21 * 2^11 and the multiply-high quotient is exact
    const uint32_t row = un.bw > 1u ? __umulhi(local, un.divBw) : local;
    const int x = un.x0 + (int)(local - row * un.bw), y = un.y0 + (int)row;
    ScreenV q[4];
    blockQuad(sh, o, q);
    const uint32_t opt = blk * HD_SEGS + wp * HD_WARP_SEGS + lo;
#pragma unroll
    for (uint32_t tr = 0; tr < 2u; tr++)
      if (x >= un.bx0[tr] && x <= un.bx1[tr] && y >= un.by0[tr] && y <= un.by1[tr])
        triPixel<WIN>(segTri(q, tr), un.area[tr], out, x, y, primOf(opt, P, tr));
  }
  if (own[0] || own[1]) {
    ScreenV q[4];
    blockQuad(sh, tid, q);
    for (uint32_t tr = 0; tr < 2u; tr++) {
      if (!own[tr]) continue;
      const Tri t = segTri(q, tr);
      float area;
      int x0, x1, y0, y1;
      if (!triBox(t, W, H, area, x0, x1, y0, y1)) continue;
      drawRows<WIN>(t, area, out, x0, x1, y0, y1, 0, 1, primOf(pt, P, tr));
    }
  }
  // the shared state is rewritten by the CTA's next points only after batchNext's barrier
}

// The big list, one block per triangle, its rows spread over the threads.
template <bool WIN>
__device__ __forceinline__ void hairDepthBigBody(const HdView& V, uint32_t P, const float4* __restrict__ pos,
                                                 const float4* __restrict__ tan, const HdOut& out,
                                                 const uint32_t* __restrict__ big, uint32_t bigCap, uint32_t blk,
                                                 uint32_t nblk) {
  const uint32_t n = bigCap ? min(*HFB_G(&big[0]), bigCap) : 0u;
  const uint32_t W = f2u(V.W), H = f2u(V.H);
  for (uint32_t e = blk; e < n; e += nblk) {
    const uint32_t ent = *HFB_G(&big[1u + e]);
    const uint32_t pt = ent >> 1, tr = ent & 1u;
    ScreenV q[4];
    pointPair(V, pos, tan, pt, q[0], q[1]);
    pointPair(V, pos, tan, (size_t)pt + 1u, q[2], q[3]);
    const Tri t = segTri(q, tr);
    float area;
    int x0, x1, y0, y1;
    if (!triBox(t, W, H, area, x0, x1, y0, y1)) continue;
    drawRows<WIN>(t, area, out, x0, x1, y0, y1, (int)threadIdx.x, (int)blockDim.x, primOf(pt, P, tr));  // row/thread
  }
}

template <bool WIN>
__global__ void __launch_bounds__(HD_THREADS, 5)
hairDepthKernel(const HdView V, uint32_t P, uint32_t nPts, const float4* __restrict__ pos,
                const float4* __restrict__ tan, const HdOut out, uint32_t* __restrict__ big, uint32_t bigCap) {
  __shared__ HdShared sh;
  hairDepthBlock<WIN>(V, P, nPts, pos, tan, out, big, bigCap, blockIdx.x, sh);
}

template <bool WIN>
__global__ void __launch_bounds__(HD_THREADS)
hairDepthBigKernel(const HdView V, uint32_t P, const float4* __restrict__ pos, const float4* __restrict__ tan,
                   const HdOut out, const uint32_t* __restrict__ big, uint32_t bigCap) {
  hairDepthBigBody<WIN>(V, P, pos, tan, out, big, bigCap, blockIdx.x, gridDim.x);
}

// ---- the hair's normals: HwHairPass's second colour output ----
// A vertex of the quad with what the fragment shader interpolates: the
// screen position, 1 / clip.w and tangentWS = modelMatrix * (tangent, 1)
// (hwHairPass.wgsl.ts:60-66, w = 1 as the reference writes it).
struct NVert {
  ScreenV s;
  float w;
  f3 t;
};

__device__ __forceinline__ NVert normalVertex(const HfbMat4& model, const HdView& V, const float4* __restrict__ pos,
                                              const float4* __restrict__ tan, size_t i, bool plus) {
  ScreenV a, b;
  pointPair(V, pos, tan, i, a, b);
  NVert n;
  n.s = plus ? a : b;
  // clip.w of the vertex, as projectScreen computed it
  const float4 p = __ldg(HFB_G(&pos[i]));
  const float4 t = __ldg(HFB_G(&tan[i]));
  const f4 pVS = m4v(V.mv, mk4(p.x, p.y, p.z, 1.0f));
  const f4 tVS = m4v(V.mv, mk4(t.x, t.y, t.z, 1.0f));
  const f3 c = cross3(xyz(tVS), mk3(0.0f, 0.0f, 1.0f));
  const f3 right = dot3(c, c) >= 1e-7f ? norm3(c) : mk3(0.0f, 0.0f, 0.0f);
  const f3 th = mul3s(right, V.radius);
  const f3 e = plus ? add3(xyz(pVS), th) : sub3(xyz(pVS), th);
  n.w = m4v(V.pr, mk4(e.x, e.y, e.z, 1.0f)).w;
  n.t = xyz(m4v(model.m, mk4(t.x, t.y, t.z, 1.0f)));
  return n;
}

// encodeOctahedronNormal (shaderSnippets.wgls.ts:25-46) of normalize(t),
// each component then stored as f16 (the rg16float target).
__device__ __forceinline__ float2 octNormal(f3 t0) {
  const f3 t = norm3(t0);
  const float s = fadd(fadd(fabsf(t.x), fabsf(t.y)), fabsf(t.z));
  float nx = t.x / s, ny = t.y / s;
  const float nz = t.z / s;
  if (nz < 0.0f) {
    const float sx = nx >= 0.0f ? 1.0f : -1.0f, sy = ny >= 0.0f ? 1.0f : -1.0f;
    const float ax = fmul(fsub(1.0f, fabsf(ny)), sx), ay = fmul(fsub(1.0f, fabsf(nx)), sy);
    nx = ax;
    ny = ay;
  }
  return make_float2(__half2float(__float2half_rn(fadd(fmul(nx, 0.5f), 0.5f))),
                     __half2float(__float2half_rn(fadd(fmul(ny, 0.5f), 0.5f))));
}

// Per pixel: the winning fragment's tangent, interpolated perspective-
// correctly (screen barycentrics b_i weighted by 1 / w_i), normalised and
// encoded; pixels without hair keep their normal.
__global__ void __launch_bounds__(256)
hairNormalResolve(const HfbMat4 model, const HdView V, uint32_t P, const float4* __restrict__ pos,
                  const float4* __restrict__ tan, const unsigned* __restrict__ winner, float2* __restrict__ normals) {
  const uint32_t W = f2u(V.W), H = f2u(V.H);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * H) return;
  const unsigned prim = __ldg(HFB_G(&winner[i]));
  if (prim == 0xFFFFFFFFu) return;
  const uint32_t tr = prim & 1u, segIdx = prim >> 1, strand = segIdx / (P - 1u), seg = segIdx - strand * (P - 1u);
  const size_t pt = (size_t)strand * P + seg;
  const NVert q[4] = {normalVertex(model, V, pos, tan, pt, true), normalVertex(model, V, pos, tan, pt, false),
                      normalVertex(model, V, pos, tan, pt + 1u, true),
                      normalVertex(model, V, pos, tan, pt + 1u, false)};
  const NVert& v0 = tr ? q[2] : q[0];
  const NVert& v1 = q[1];
  const NVert& v2 = tr ? q[3] : q[2];
  const float px = fadd((float)(i % W), 0.5f), py = fadd((float)(i / W), 0.5f);
  const float area = edgeFn(v0.s.x, v0.s.y, v1.s.x, v1.s.y, v2.s.x, v2.s.y);
  float b0 = edgeFn(v1.s.x, v1.s.y, v2.s.x, v2.s.y, px, py);
  float b1 = edgeFn(v2.s.x, v2.s.y, v0.s.x, v0.s.y, px, py);
  float b2 = edgeFn(v0.s.x, v0.s.y, v1.s.x, v1.s.y, px, py);
  if (area < 0.0f) { b0 = -b0; b1 = -b1; b2 = -b2; }
  const float a = fabsf(area);
  const float p0 = (b0 / a) / v0.w, p1 = (b1 / a) / v1.w, p2 = (b2 / a) / v2.w;
  const float sum = fadd(fadd(p0, p1), p2);
  const f3 t = mk3(fadd(fadd(fmul(p0, v0.t.x), fmul(p1, v1.t.x)), fmul(p2, v2.t.x)) / sum,
                   fadd(fadd(fmul(p0, v0.t.y), fmul(p1, v1.t.y)), fmul(p2, v2.t.y)) / sum,
                   fadd(fadd(fmul(p0, v0.t.z), fmul(p1, v1.t.z)), fmul(p2, v2.t.z)) / sum);
  *HFB_G(&normals[i]) = octNormal(t);
}

// The instance's HdView into shared memory (every thread calls; synced).
__device__ __forceinline__ void loadView(const HfbUniforms& U, HdView& V) {
  __syncthreads();  // the previous instance's view is no longer read
  if (threadIdx.x < HD_VIEW_FLOATS) reinterpret_cast<float*>(&V)[threadIdx.x] = hdViewField(U, threadIdx.x);
  __syncthreads();
}

// ---- batched: persistent over every instance ----
// 5 blocks per SM (48 registers): 1.33 ms against 1.40 at 4 on the 64-instance frame
__global__ void __launch_bounds__(HD_THREADS, 5) hairDepthBatch(BatchView b) {
  __shared__ HdShared sh;
  __shared__ HdView V;
  const uint32_t n = b.hdr->n;
  const uint32_t* row = b.prefix + BK_HAIR_DEPTH * (BATCH_MAX + 1);
  const uint32_t total = row[n];
  uint32_t cur = 0xFFFFFFFFu;
  __shared__ uint32_t vbNext[2];
  uint32_t vbPar = 0;
  for (uint32_t v = batchNext(b.hdr, BK_HAIR_DEPTH, vbNext, vbPar); v < total; v = batchNext(b.hdr, BK_HAIR_DEPTH, vbNext, vbPar)) {
    const uint32_t i = batchFind(row, n, v);
    const BatchInst& I = b.insts[i];
    if (i != cur) {
      loadView(I.U, V);
      cur = i;
    }
    const HdOut out = {reinterpret_cast<unsigned*>(I.hairDepth), nullptr, I.W};
    hairDepthBlock<false>(V, I.P, min(I.strandsToRender, I.S) * I.P, I.posNew, I.tan, out, I.hdList, I.hdCap,
                          v - row[i], sh);
  }
}

__global__ void __launch_bounds__(HD_THREADS) hairDepthBigBatch(BatchView b) {
  __shared__ HdView V;
  const uint32_t n = b.hdr->n;
  for (uint32_t i = 0; i < n; i++) {  // every block takes a share of each instance's list
    const BatchInst& I = b.insts[i];
    if (!I.hairDepth) continue;
    loadView(I.U, V);
    const HdOut out = {reinterpret_cast<unsigned*>(I.hairDepth), nullptr, I.W};
    hairDepthBigBody<false>(V, I.P, I.posNew, I.tan, out, I.hdList, I.hdCap, blockIdx.x, gridDim.x);
  }
}

}  // namespace

uint32_t hairDepthBlocks(uint32_t points) { return divCeil(points, HD_SEGS); }

cudaError_t launchHairDepth(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h, const float* pos, const float* tan,
                            uint32_t strandsToRender, const float* sceneDepth, float* hairDepth,
                            HfbRasterBuffers& rb) {
  HFB_CHECK_BIND(c);
  const size_t px = (size_t)rb.width * rb.height;
  uint32_t cap = 0;
  uint32_t* big = hairDepthList(rb.scratch, rb.scratchBytes,
                                rasterPassScratchBytes(c->cfg, rb.width, rb.height, rb.maxDrawnSegments), &cap);
  cudaError_t e = cudaMemcpyAsync(hairDepth, sceneDepth, px * 4, cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess && big) e = cudaMemsetAsync(big, 0, 4, c->stream);  // the big list's count
  if (e != cudaSuccess) return e;
  const uint32_t nStrands = min(strandsToRender, h.strandsCount);
  const uint32_t nPts = nStrands * h.pointsPerStrand;
  if (h.pointsPerStrand < 2u || nPts == 0) return cudaSuccess;
  const HdView V = hdView(u);
  const HdOut out = {(unsigned*)hairDepth, nullptr, rb.width};
  hairDepthKernel<false><<<hairDepthBlocks(nPts), HD_THREADS, 0, c->stream>>>(
      V, h.pointsPerStrand, nPts, (const float4*)pos, (const float4*)tan, out, big, cap);
  HFB_AFTER_LAUNCH(c, "hairDepthKernel");
  hairDepthBigKernel<false><<<c->smCount * 4u, HD_THREADS, 0, c->stream>>>(
      V, h.pointsPerStrand, (const float4*)pos, (const float4*)tan, out, big, cap);
  HFB_AFTER_LAUNCH(c, "hairDepthBigKernel");
  c->launches += 2;
  return cudaGetLastError();
}

cudaError_t launchHairNormals(HfbCtx* c, const HfbUniforms& u, const HfbHairData& h,
                              const float* pos, const float* tan, uint32_t strandsToRender, const float* hairDepth,
                              float* normals, uint32_t* winner, HfbRasterBuffers& rb) {
  HFB_CHECK_BIND(c);
  const size_t px = (size_t)rb.width * rb.height;
  uint32_t cap = 0;
  uint32_t* big = hairDepthList(rb.scratch, rb.scratchBytes,
                                rasterPassScratchBytes(c->cfg, rb.width, rb.height, rb.maxDrawnSegments), &cap);
  cudaError_t e = cudaMemsetAsync(winner, 0xFF, px * 4, c->stream);
  if (e == cudaSuccess && big) e = cudaMemsetAsync(big, 0, 4, c->stream);
  if (e != cudaSuccess) return e;
  const uint32_t nStrands = min(strandsToRender, h.strandsCount);
  const uint32_t nPts = nStrands * h.pointsPerStrand;
  if (h.pointsPerStrand < 2u || nPts == 0) return cudaSuccess;
  const HdView V = hdView(u);
  const HdOut out = {(unsigned*)hairDepth, winner, rb.width};
  hairDepthKernel<true><<<hairDepthBlocks(nPts), HD_THREADS, 0, c->stream>>>(
      V, h.pointsPerStrand, nPts, (const float4*)pos, (const float4*)tan, out, big, cap);
  HFB_AFTER_LAUNCH(c, "hairDepthKernel<winner>");
  hairDepthBigKernel<true><<<c->smCount * 4u, HD_THREADS, 0, c->stream>>>(
      V, h.pointsPerStrand, (const float4*)pos, (const float4*)tan, out, big, cap);
  HFB_AFTER_LAUNCH(c, "hairDepthBigKernel<winner>");
  hairNormalResolve<<<divCeil((uint32_t)px, 256u), 256, 0, c->stream>>>(
      u.modelMatrix, V, h.pointsPerStrand, (const float4*)pos, (const float4*)tan, winner, (float2*)normals);
  HFB_AFTER_LAUNCH(c, "hairNormalResolve");
  c->launches += 3;
  return cudaGetLastError();
}

cudaError_t launchBatchHairDepth(HfbCtx* c, const BatchView& b) {
  HFB_CHECK_BIND(c);
  uint32_t& grid = c->batchGrid[BK_HAIR_DEPTH];
  if (!grid) grid = c->smCount * 8u;
  hairDepthBatch<<<batchLaunchGrid(c, grid), HD_THREADS, 0, c->stream>>>(b);
  HFB_AFTER_LAUNCH(c, "hairDepthBatch");
  hairDepthBigBatch<<<batchLaunchGrid(c, c->smCount * 4u), HD_THREADS, 0, c->stream>>>(b);
  HFB_AFTER_LAUNCH(c, "hairDepthBigBatch");
  c->launches += 2;
  return cudaGetLastError();
}

}  // namespace hfb
