"""ctypes bindings of libhairfb.so (include/hairfb.h).

The library is the only compute path: if it is missing or does not load,
every entry point here raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .config import HfbConfig

# HAIRFB_LIBRARY selects another build of the library (e.g. the self-checking one)
LIB_PATH = os.environ.get("HAIRFB_LIBRARY") or \
    os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libhairfb.so")

HFB_OK = 0
HFB_ERR_INVALID_ARGUMENT = -1
HFB_ERR_OUT_OF_MEMORY = -2
HFB_ERR_CUDA = -3
HFB_ERR_UNSUPPORTED = -6


class HfbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hairfb error {code}: {msg}")
        self.code = code


class HfbHairData(ctypes.Structure):
    _fields_ = [("boundingSphere", ctypes.c_float * 4), ("strandsCount", ctypes.c_uint32),
                ("pointsPerStrand", ctypes.c_uint32), ("padding", ctypes.c_uint32 * 2)]


class HfbRasterBuffers(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("maxDrawnSegments", ctypes.c_uint32), ("reserved0", ctypes.c_uint32),
                ("tiles", ctypes.c_void_p), ("tileSegments", ctypes.c_void_p),
                ("segmentCountPerTile", ctypes.c_void_p), ("sortBuckets", ctypes.c_void_p),
                ("tileList", ctypes.c_void_p), ("rasterizerResult", ctypes.c_void_p),
                ("scratch", ctypes.c_void_p), ("scratchBytes", ctypes.c_size_t)]


class HfbPresentItem(ctypes.Structure):
    """One hfb_present call's arguments, for hfb_present_batch (host
    addresses of the uniforms and the raster buffers' struct, device
    addresses of the scene colour (or NULL) and the RGBA8 image)."""
    _fields_ = [("uniforms", ctypes.c_void_p), ("rb", ctypes.c_void_p), ("sceneColor", ctypes.c_void_p),
                ("rgba", ctypes.c_void_p)]


class HfbInstance(ctypes.Structure):
    """One hair instance of a frame (hfb_frame / hfb_frame_batch)."""
    _fields_ = [("uniforms", ctypes.c_void_p), ("simUniforms", ctypes.c_void_p), ("hair", HfbHairData),
                ("positions", ctypes.c_void_p * 2), ("current", ctypes.c_uint32),
                ("strandsToRender", ctypes.c_uint32), ("positionsInitial", ctypes.c_void_p),
                ("tangents", ctypes.c_void_p), ("segmentLengths", ctypes.c_void_p),
                ("densityVelocity", ctypes.c_void_p), ("densityGradWind", ctypes.c_void_p),
                ("sdf", ctypes.c_void_p), ("sdfDims", ctypes.c_uint32), ("shadowMapSize", ctypes.c_uint32),
                ("shading", ctypes.c_void_p), ("sceneDepth", ctypes.c_void_p), ("shadingDepth", ctypes.c_void_p),
                ("ao", ctypes.c_void_p), ("aoWidth", ctypes.c_uint32), ("aoHeight", ctypes.c_uint32),
                ("shadowMap", ctypes.c_void_p), ("raster", HfbRasterBuffers), ("hairDepth", ctypes.c_void_p),
                ("gridOrder", ctypes.c_void_p)]


class HfbCounters(ctypes.Structure):
    _fields_ = [("tileRecords", ctypes.c_uint64), ("tileRecordsDropped", ctypes.c_uint64),
                ("finePoolFullBins", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("fineSplitTiles", ctypes.c_uint64),
                ("fineSplitRedone", ctypes.c_uint64), ("badWorkItems", ctypes.c_uint64)]


assert ctypes.sizeof(HfbHairData) == 32
assert ctypes.sizeof(HfbCounters) == 56
assert ctypes.sizeof(HfbInstance) == 272

# every symbol include/hairfb.h declares: name -> (restype, argtypes)
P, U32, SZ, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_size_t, ctypes.c_int
SIGNATURES = {
    "hfb_version": (I, []),
    "hfb_ctx_create": (I, [P, I, P]),
    "hfb_ctx_destroy": (I, [P]),
    "hfb_last_error": (ctypes.c_char_p, [P]),
    "hfb_ctx_set_stream": (I, [P, P]),
    "hfb_sync": (I, [P]),
    "hfb_get_counters": (I, [P, P]),
    "hfb_check_constant_division": (I, [P, P]),
    "hfb_buffer_alloc": (I, [P, SZ, P]),
    "hfb_buffer_free": (I, [P, P]),
    "hfb_buffer_upload": (I, [P, P, P, SZ]),
    "hfb_buffer_download": (I, [P, P, P, SZ]),
    "hfb_buffer_clear": (I, [P, P, SZ]),
    "hfb_raster_scratch_bytes": (SZ, [P, U32, U32]),
    "hfb_raster_scratch_bytes_for": (SZ, [P, U32, U32, U32]),
    "hfb_raster_buffers_alloc_sized": (I, [P, U32, U32, U32, P]),
    "hfb_raster_buffers_alloc": (I, [P, U32, U32, P]),
    "hfb_raster_buffers_free": (I, [P, P]),
    "hfb_grid_pre_sim": (I, [P, P, P, P, P, U32]),
    "hfb_sim_integrate": (I, [P, P, P, P, P, P, P, P, P, P, U32]),
    "hfb_grid_post_sim": (I, [P, P, P, P, P, P]),
    "hfb_grid_post_sim_ordered": (I, [P, P, P, P, P, P, P]),
    "hfb_strand_grid_order": (I, [P, U32, U32, P]),
    "hfb_shading": (I, [P, P, P, P, P, P, P, U32, U32, P, U32, P]),
    "hfb_clear_before_render": (I, [P, P]),
    "hfb_tiles_pass": (I, [P, P, P, P, P, P, U32, P]),
    "hfb_tile_sort": (I, [P, P]),
    "hfb_fine_pass": (I, [P, P, P, P, P, P, P, P]),
    "hfb_tiles_pass_noalloc": (I, [P, P, P, P, P, P, U32, P]),
    "hfb_hair_depth": (I, [P, P, P, P, P, U32, P, P, P]),
    "hfb_present": (I, [P, P, P, P, P]),
    "hfb_present_batch": (I, [P, P, U32]),
    "hfb_hair_normals": (I, [P, P, P, P, P, U32, P, P, P, P]),
    "hfb_gtao": (I, [P, P, P, P, ctypes.c_float, P]),
    "hfb_frame": (I, [P, P]),
    "hfb_frame_batch": (I, [P, P, U32]),
    "hfb_frame_batch_profile": (I, [P, P, U32, P]),
    "hfb_ctx_set_batch_groups": (I, [P, U32]),
    "hfb_ctx_set_batch_pipeline": (I, [P, U32]),
}

_lock = threading.Lock()
_lib = None


def open_library(path: str):
    """Opens a libhairfb.so and declares every entry point; raises if it is
    absent (no fallback path exists)."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: build it with `python -m hairfb.build` (needs nvcc)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load(path: str = LIB_PATH):
    """The process-wide libhairfb.so."""
    global _lib
    with _lock:
        if _lib is None:
            _lib = open_library(path)
    return _lib


def strand_grid_order(positions, strands: int, points: int):
    """hfb_strand_grid_order: the strands sorted by their root's Morton code
    (a uint32 numpy array), the order the grid splat visits them in."""
    import numpy as np
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    assert pos.size >= strands * points * 4
    out = np.empty(strands, np.uint32)
    rc = load().hfb_strand_grid_order(pos.ctypes.data, strands, points, out.ctypes.data)
    if rc != HFB_OK:
        raise HfbError(rc, "hfb_strand_grid_order failed")
    return out


def ptr(x) -> int | None:
    """Device address of a torch tensor (or pass-through int / None)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def byref(s):
    return ctypes.cast(ctypes.pointer(s), ctypes.c_void_p)


class Context:
    """Owns one HfbCtx (a CUDA stream + the pass constants)."""

    def __init__(self, cfg: HfbConfig, device: int = -1):
        self.lib = load()
        self.cfg = cfg
        h = ctypes.c_void_p()
        rc = self.lib.hfb_ctx_create(byref(cfg), device, ctypes.byref(h))
        if rc != HFB_OK:
            raise HfbError(rc, "hfb_ctx_create failed (invalid config or CUDA error)")
        self.handle = h

    def check(self, rc: int) -> None:
        if rc != HFB_OK:
            msg = self.lib.hfb_last_error(self.handle)
            raise HfbError(rc, msg.decode() if msg else "")

    def call(self, name: str, *args) -> None:
        self.check(getattr(self.lib, name)(self.handle, *args))

    def set_stream(self, stream) -> None:
        """Run on a torch.cuda.Stream (or raw cudaStream_t int); None = the
        context's own stream.  Handle 0 (torch's default stream) is the
        legacy default stream, passed as cudaStreamLegacy."""
        self.stream_obj = stream
        if stream is None:
            self.call("hfb_ctx_set_stream", None)
            return
        h = stream if isinstance(stream, int) else stream.cuda_stream
        self.call("hfb_ctx_set_stream", h if h else 1)  # 1 == cudaStreamLegacy

    def sync(self) -> None:
        self.call("hfb_sync")

    def set_batch_groups(self, groups: int) -> None:
        """hfb_frame_batch runs its instances in `groups` groups side by side."""
        self.call("hfb_ctx_set_batch_groups", groups)
        self.batch_groups = groups

    def set_batch_pipeline(self, on: bool) -> None:
        """hfb_frame_batch overlaps a frame's simulation with the previous
        frame's raster passes (see hfb_ctx_set_batch_pipeline)."""
        self.call("hfb_ctx_set_batch_pipeline", 1 if on else 0)
        self.batch_pipeline = bool(on)

    def counters(self) -> dict:
        c = HfbCounters()
        self.call("hfb_get_counters", byref(c))
        return {k: getattr(c, k) for k, _ in HfbCounters._fields_ if k != "reserved"}

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.hfb_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
