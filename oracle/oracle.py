"""TEST INFRASTRUCTURE -- ctypes front end of the CPU oracle.

Builds ``oracle/_build/libhairfb_oracle.so`` from ``hairfb_oracle.c`` (gcc,
``-O2 -ffp-contract=off``) and exposes one numpy function per reference pass.
Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hairfb_oracle.c")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libhairfb_oracle.so")
LIB_OMP = os.path.join(BUILD, "libhairfb_oracle_omp.so")

_lock = threading.Lock()
_libs = {}
_threaded = False

CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-Wall", "-Wno-unknown-pragmas"]


def _build_one(out: str, extra, force: bool) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(SRC):
        tmp = out + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", *CFLAGS, *extra, "-o", tmp, SRC, "-lm"])
        os.replace(tmp, out)
    return out


def build(force: bool = False) -> str:
    """Compile both builds of the oracle: serial (the canonical checker) and
    OpenMP (the same arithmetic on every host core, for the CPU baseline)."""
    _build_one(LIB_OMP, ["-fopenmp"], force)
    return _build_one(LIB, [], force)


def use_threads(on: bool) -> None:
    """Route subsequent calls to the OpenMP build (True) or the serial one."""
    global _threaded
    _threaded = bool(on)


def load(threaded: bool | None = None):
    t = _threaded if threaded is None else threaded
    with _lock:
        if t not in _libs:
            build()
            lib = ctypes.CDLL(LIB_OMP if t else LIB)
            _declare(lib)
            _libs[t] = lib
    return _libs[t]


def _declare(lib):
    P = ctypes.c_void_p
    U = ctypes.c_uint32
    lib.oracle_sw_raster_test.argtypes = [P, P, P, P, P]
    lib.oracle_tiles_pass.argtypes = [P, P, P, P, P, P, U, P, P, P]
    lib.oracle_tile_sort.argtypes = [P, U, U, P, P, P]
    lib.oracle_fine_pass.argtypes = [P, P, P, P, P, P, P, P, P, P, P]
    lib.oracle_grid_pre_sim.argtypes = [P, P, P, P, U, P]
    lib.oracle_sim_integrate.argtypes = [P, P, P, P, P, P, P, P, P, P, U]
    lib.oracle_grid_post_sim.argtypes = [P, P, P, P, P, P]
    lib.oracle_shading.argtypes = [P, P, P, P, P, P, P, U, U, P, U, P]
    lib.oracle_hair_depth.argtypes = [P, P, P, P, U, P]
    lib.oracle_present.argtypes = [P, P, P, P]
    lib.oracle_hair_normals.argtypes = [P, P, P, P, U, P, P]
    lib.oracle_gtao.argtypes = [P, P, P, ctypes.c_float, P]
    lib.oracle_sample_sdf.argtypes = [P, U, P, P, P]
    lib.oracle_sample_sdf.restype = ctypes.c_float
    lib.oracle_f32_to_f16.argtypes = [ctypes.c_float]
    lib.oracle_f32_to_f16.restype = ctypes.c_uint16
    lib.oracle_f16_to_f32.argtypes = [ctypes.c_uint16]
    lib.oracle_f16_to_f32.restype = ctypes.c_float


def _p(a):
    if a is None:
        return None
    if isinstance(a, (bytes, bytearray)):
        return ctypes.cast(ctypes.c_char_p(bytes(a)), ctypes.c_void_p)
    if isinstance(a, ctypes.Structure):
        return ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be contiguous"
    return ctypes.c_void_p(a.ctypes.data)


class _Bytes:
    """Keeps a bytes object alive while a pointer to it is in use."""

    def __init__(self, b: bytes):
        self.buf = ctypes.create_string_buffer(bytes(b), len(b))

    @property
    def ptr(self):
        return ctypes.cast(self.buf, ctypes.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# --------------------------------------------------------------------------
# passes
# --------------------------------------------------------------------------

def sw_raster_test(uniforms: bytes, hair_data: bytes, positions, tangents, width, height):
    lib = load()
    out = np.zeros(width * height, np.uint32)
    u, h = _Bytes(uniforms), _Bytes(hair_data)
    lib.oracle_sw_raster_test(u.ptr, h.ptr, _p(_f32(positions)), _p(_f32(tangents)), _p(out))
    return out


def tiles_pass(cfg, uniforms: bytes, hair_data: bytes, positions, tangents, depth,
               strands_to_render, width, height, max_drawn):
    """Returns (tiles[T*B,4] u32, segments[1 + 2*maxDrawn] u32, seg_count[T] u32)."""
    lib = load()
    tx, ty = cfg.tile_count(width, height)
    T = tx * ty
    tiles = np.zeros((T * cfg.tile_depth_bins, 4), np.uint32)
    segs = np.zeros(1 + 2 * max_drawn, np.uint32)
    cnt = np.zeros(T, np.uint32)
    c = cfg.to_c()
    u, h = _Bytes(uniforms), _Bytes(hair_data)
    lib.oracle_tiles_pass(_p(c), u.ptr, h.ptr, _p(_f32(positions)), _p(_f32(tangents)),
                          _p(_f32(depth)), strands_to_render, _p(tiles), _p(segs), _p(cnt))
    return tiles, segs, cnt


def tile_sort(cfg, width, height, seg_count):
    lib = load()
    tx, ty = cfg.tile_count(width, height)
    buckets = np.zeros(2 * cfg.sort_buckets, np.uint32)
    tile_list = np.zeros(4 + tx * ty, np.uint32)
    c = cfg.to_c()
    lib.oracle_tile_sort(_p(c), width, height, _p(np.ascontiguousarray(seg_count, np.uint32)),
                         _p(buckets), _p(tile_list))
    return buckets, tile_list


def fine_pass(cfg, uniforms: bytes, hair_data: bytes, positions, tangents, shading, depth,
              tiles, segs, tile_list, width, height):
    lib = load()
    result = np.zeros(4 + 4 * width * height, np.float32)
    c = cfg.to_c()
    u, h = _Bytes(uniforms), _Bytes(hair_data)
    lib.oracle_fine_pass(_p(c), u.ptr, h.ptr, _p(_f32(positions)), _p(_f32(tangents)),
                         _p(_f32(shading)), _p(_f32(depth)),
                         _p(np.ascontiguousarray(tiles, np.uint32)),
                         _p(np.ascontiguousarray(segs, np.uint32)),
                         _p(np.ascontiguousarray(tile_list, np.uint32)), _p(result))
    return result


def grid_pre_sim(cfg, sim_uniforms: bytes, dens_vel, sdf, sdf_dims):
    lib = load()
    G = cfg.grid_dims
    out = np.zeros((G * G * G, 4), np.float32)
    c = cfg.to_c()
    u = _Bytes(sim_uniforms)
    lib.oracle_grid_pre_sim(_p(c), u.ptr, _p(np.ascontiguousarray(dens_vel, np.int32)),
                            _p(_f32(sdf)), sdf_dims, _p(out))
    return out


def sim_integrate(cfg, sim_uniforms: bytes, hair_data: bytes, prev, now, initial, seg_lengths,
                  dens_vel, grad_wind, sdf, sdf_dims):
    """Returns the new positions (written into a copy of ``prev``)."""
    lib = load()
    out = _f32(prev).copy()
    c = cfg.to_c()
    u, h = _Bytes(sim_uniforms), _Bytes(hair_data)
    lib.oracle_sim_integrate(_p(c), u.ptr, h.ptr, _p(out), _p(_f32(now)), _p(_f32(initial)),
                             _p(_f32(seg_lengths)), _p(np.ascontiguousarray(dens_vel, np.int32)),
                             _p(_f32(grad_wind)), _p(_f32(sdf)), sdf_dims)
    return out


def grid_post_sim(cfg, sim_uniforms: bytes, hair_data: bytes, prev, now):
    lib = load()
    G = cfg.grid_dims
    out = np.zeros((G * G * G, 4), np.int32)
    c = cfg.to_c()
    u, h = _Bytes(sim_uniforms), _Bytes(hair_data)
    lib.oracle_grid_post_sim(_p(c), u.ptr, h.ptr, _p(_f32(prev)), _p(_f32(now)), _p(out))
    return out


def hair_depth(uniforms: bytes, hair_data: bytes, positions, tangents, strands_to_render, scene_depth):
    """HwHairPass's depth: scene_depth (W*H) with the hair drawn over it."""
    lib = load()
    out = np.array(scene_depth, dtype=np.float32, copy=True).reshape(-1)
    u, h = _Bytes(uniforms), _Bytes(hair_data)
    lib.oracle_hair_depth(u.ptr, h.ptr, _p(_f32(positions)), _p(_f32(tangents)), strands_to_render, _p(out))
    return out


def hair_normals(uniforms: bytes, hair_data: bytes, positions, tangents, strands_to_render, hair_depth,
                 normals=None):
    """HwHairPass's normal output: (W*H, 2) float32 (f16 values), pixels
    without hair keep `normals` (zeros when None)."""
    lib = load()
    u, h = _Bytes(uniforms), _Bytes(hair_data)
    hd = _f32(hair_depth).reshape(-1)
    out = np.zeros((hd.size, 2), np.float32) if normals is None else np.array(normals, np.float32, copy=True)
    lib.oracle_hair_normals(u.ptr, h.ptr, _p(_f32(positions)), _p(_f32(tangents)), strands_to_render, _p(hd),
                            _p(out))
    return out


def gtao(uniforms: bytes, depth, normals, scale=0.5):
    """AoPass: (ceil(H*scale), ceil(W*scale)) float32 (f16 values)."""
    import math
    lib = load()
    u = _Bytes(uniforms)
    vp = np.frombuffer(uniforms, np.float32)[16 * 9:16 * 9 + 2]
    aw, ah = math.ceil(float(vp[0]) * scale), math.ceil(float(vp[1]) * scale)
    out = np.zeros(aw * ah, np.float32)
    lib.oracle_gtao(u.ptr, _p(_f32(depth).reshape(-1)), _p(_f32(normals).reshape(-1)), scale, _p(out))
    return out.reshape(ah, aw)


def present(uniforms: bytes, result, scene_color=None):
    """HairCombinePass + PresentPass: result = the W*H vec4f pixels of the
    fine pass (without the header), scene_color W*H vec4f or None; returns
    (H, W, 4) uint8, row 0 at the top."""
    lib = load()
    u = _Bytes(uniforms)
    res = _f32(result)
    n = res.size // 4
    out = np.zeros(n * 4, np.uint8)
    sc = _f32(scene_color) if scene_color is not None else None
    lib.oracle_present(u.ptr, _p(res), _p(sc) if sc is not None else None, out.ctypes.data)
    W = int(round(np.frombuffer(uniforms, np.float32)[16 * 9]))
    return out.reshape(-1, W, 4)


def shading(cfg, uniforms: bytes, hair_data: bytes, positions, tangents, depth, strands,
            ao=None, ao_size=(0, 0), shadow_map=None, shadow_size=0):
    lib = load()
    out = np.zeros((strands * cfg.shading_points, 4), np.float32)
    c = cfg.to_c()
    u, h = _Bytes(uniforms), _Bytes(hair_data)
    lib.oracle_shading(_p(c), u.ptr, h.ptr, _p(_f32(positions)), _p(_f32(tangents)),
                       _p(_f32(depth)), _p(None if ao is None else _f32(ao)),
                       ao_size[0], ao_size[1],
                       _p(None if shadow_map is None else _f32(shadow_map)), shadow_size, _p(out))
    return out


def sample_sdf(sdf, dims, bmin, bmax, p):
    lib = load()
    return lib.oracle_sample_sdf(_p(_f32(sdf)), dims, _p(_f32(bmin)), _p(_f32(bmax)), _p(_f32(p)))


# --------------------------------------------------------------------------
# helpers for comparing the reference-layout list buffers
# --------------------------------------------------------------------------

INVALID = 0xFFFFFFFF


def walk_lists(tiles, segs, max_drawn):
    """Walk every per-(tile, depth bin) linked list from its head.
    Returns {tileBinIdx: [encoded (seg << 24 | strand), ...]} in list order."""
    out = {}
    data = segs[1:].reshape(-1, 2)
    heads = tiles[:, 2]
    for tb in np.nonzero(heads)[0]:
        ptr = int(heads[tb]) - 1
        seq = []
        steps = 0
        while ptr != INVALID and ptr < max_drawn:
            seq.append(int(data[ptr, 0]))
            ptr = int(data[ptr, 1])
            steps += 1
            if steps > data.shape[0]:
                raise RuntimeError("cycle in a tile segment list")
        out[int(tb)] = seq
    return out
