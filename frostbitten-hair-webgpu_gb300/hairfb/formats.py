"""Asset file formats the reference loads: TFX hair and the binary SDF.

- TFX: ``parseTfxFile`` (src/scene/hair/tfxFileLoader.ts:19-69). Header:
  f32 version, then u32 numHairStrands, numVerticesPerStrand,
  offsetVertexPosition, offsetStrandUV, offsetVertexUV, offsetStrandThickness,
  offsetVertexColor, then 32 reserved u32 (160 bytes in total, as the Blender
  exporter writes it, scripts/tfx_exporter.py); positions are
  FLOAT4[strands * vertsPerStrand] at offsetVertexPosition.
- SDF: ``createSdfColliderFromBinary``
  (src/scene/sdfCollider/createSdfColliderFromBinary.ts:5-43): u32 dims,
  4 ignored bytes, 6 f32 bounds (min xyz, max xyz), then dims^3 f32 distances,
  x fastest.

Malformed files raise ``ValueError`` (the reference throws ``Error``).
"""
from __future__ import annotations

import dataclasses
import struct

import numpy as np

from .hair_object import HairAsset

TFX_HEADER_BYTES = 160


def parse_tfx(data: bytes, scale: float = 1.0) -> HairAsset:
    if len(data) < 32:
        raise ValueError(f"Invalid TFX file: {len(data)} bytes is shorter than the header")
    version = struct.unpack_from("<f", data, 0)[0]
    (strands, verts, off_pos, _suv, _vuv, _thick, _col) = struct.unpack_from("<7I", data, 4)
    del version
    n = strands * verts * 4
    if strands == 0 or verts < 2:
        raise ValueError(f"Invalid TFX file: {strands} strands x {verts} vertices")
    if off_pos + n * 4 > len(data) or off_pos % 4:
        raise ValueError(f"Invalid TFX file: positions at {off_pos} overrun {len(data)} bytes")
    pos = np.frombuffer(data, dtype=np.float32, count=n, offset=off_pos).copy()
    if scale != 1.0:
        pos = (pos.astype(np.float64) * scale).astype(np.float32)
    return HairAsset(strands, verts, pos.reshape(-1, 4))


def write_tfx(asset: HairAsset) -> bytes:
    hdr = bytearray(TFX_HEADER_BYTES)
    struct.pack_into("<f7I", hdr, 0, 4.0, asset.strands, asset.points_per_strand,
                     TFX_HEADER_BYTES, 0, 0, 0, 0)
    return bytes(hdr) + np.ascontiguousarray(asset.positions, dtype=np.float32).tobytes()


@dataclasses.dataclass
class SdfVolume:
    dims: int
    bounds_min: np.ndarray
    bounds_max: np.ndarray
    distances: np.ndarray  # (dims^3,) float32, x fastest, then y, then z


def parse_sdf(data: bytes) -> SdfVolume:
    if len(data) < 32:
        raise ValueError(f"Invalid SDF binary file: {len(data)} bytes")
    dims = struct.unpack_from("<I", data, 0)[0]
    f = np.frombuffer(data, dtype=np.float32, count=(len(data) // 4))
    bmin = f[2:5].copy()
    bmax = f[5:8].copy()
    dist = f[8:].copy()
    exp = dims * dims * dims
    if dist.shape[0] != exp:
        raise ValueError(f"Invalid SDF binary file. With dims={dims} expected {exp} values. "
                         f"Got {dist.shape[0]}.")
    return SdfVolume(dims, bmin, bmax, dist)


def write_sdf(vol: SdfVolume) -> bytes:
    hdr = struct.pack("<II", vol.dims, 0)
    b = np.concatenate([np.asarray(vol.bounds_min, np.float32), np.asarray(vol.bounds_max, np.float32)])
    return hdr + b.tobytes() + np.ascontiguousarray(vol.distances, np.float32).tobytes()


def write_png(rgba) -> bytes:
    """An (H, W, 4) uint8 image as PNG bytes (8-bit RGBA, no filtering)."""
    import zlib
    img = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = img.shape[:2]
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
