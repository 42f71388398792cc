"""Seeded synthetic workloads with the shapes of the benchmark configurations.

There is no public dataset for this path; these generators stand in for the
Sintel asset with the sizes and distributions of the five workloads:

- ``plain_small``  2,000 x 16 strands, 640x480, tiles 16, 8 depth bins, 4 slices
- ``plain_full``   10,000 x 32 curly strands, 1920x1080, 16 bins, 4 slices, wind
- ``batched``      64 instances, 1k-20k strands, 16/24/32 points, 256^2..1024^2
- ``served``       sessions with 500-50k strands, 32 points, 256^2..2048^2
- ``stress``       200,000 x 32 strands, 60% in a ponytail cone, 3840x2160

Growth model: roots uniform on the upper hemisphere of a head sphere of
radius 0.1 (normal = radial), fixed segment length 0.01, every segment
direction = the previous one rotated by N(0, 0.2 rad) about a random
perpendicular axis; root ``w = 0``, all other points ``w = 1``.
Camera: fov 30 deg, near 0.01, far 100, looking at the hair bounding-sphere
centre from +z so the sphere fills ~80% of the viewport height.
The scene depth (the reference's mesh pass) is the head sphere at 0.98 of
its radius, written as NDC depth in a ``depth24plus``-like f32 buffer.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import matrices as M
from .config import HairConfig, SimulationParams
from .formats import SdfVolume
from .hair_object import HairAsset, build_hair_buffers, HairBuffers, scale_bounding_box
from .uniforms import Camera, SceneParams


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def _random_perp(rng, d):
    a = rng.standard_normal(d.shape)
    a = a - np.sum(a * d, axis=-1, keepdims=True) * d
    return _unit(a)


def grow_hair(rng: np.random.Generator, strands: int, points: int, *, center=(0.0, 0.0, 0.0),
              head_radius: float = 0.1, seg_len: float = 0.01, sigma: float = 0.2,
              curl: bool = False, ponytail_fraction: float = 0.0) -> HairAsset:
    c = np.asarray(center, np.float64)
    y = rng.uniform(0.0, 1.0, strands)
    phi = rng.uniform(0.0, 2.0 * math.pi, strands)
    s = np.sqrt(np.maximum(0.0, 1.0 - y * y))
    n = np.stack([s * np.cos(phi), y, s * np.sin(phi)], axis=-1)
    d = n.copy()
    sig = np.full(strands, sigma)
    n_tail = int(round(ponytail_fraction * strands))
    if n_tail:
        # ponytail: roots in a cap at the back of the head, growing down a cone
        axis = _unit(np.array([0.0, 0.35, -1.0]))
        cap = _unit(axis + 0.25 * rng.standard_normal((n_tail, 3)))
        n[:n_tail] = cap
        cone = _unit(np.array([0.0, -1.0, -0.35]))
        d[:n_tail] = _unit(cone + 0.08 * rng.standard_normal((n_tail, 3)))
        sig[:n_tail] = 0.05
    pos = np.zeros((strands, points, 4), np.float64)
    p = c + head_radius * n
    pos[:, 0, :3] = p
    e1 = _random_perp(rng, n)
    e2 = np.cross(n, e1)
    phase = rng.uniform(0.0, 2.0 * math.pi, strands)
    for k in range(1, points):
        ang = rng.standard_normal(strands) * sig
        u = _random_perp(rng, d)
        d = _unit(np.cos(ang)[:, None] * d + np.sin(ang)[:, None] * u)
        if curl:
            a = phase + 0.8 * k
            d = _unit(d + 0.3 * (np.cos(a)[:, None] * e1 + np.sin(a)[:, None] * e2))
        p = p + seg_len * d
        pos[:, k, :3] = p
    pos[:, 1:, 3] = 1.0
    return HairAsset(strands, points, pos.reshape(-1, 4).astype(np.float32))


def sdf_from_function(fn, dims: int, bmin, bmax) -> SdfVolume:
    """Distances at texel centres ((i + 0.5) / dims of the bounds), x fastest."""
    bmin = np.asarray(bmin, np.float64)
    bmax = np.asarray(bmax, np.float64)
    t = (np.arange(dims) + 0.5) / dims
    zs, ys, xs = np.meshgrid(t, t, t, indexing="ij")
    p = bmin + np.stack([xs, ys, zs], axis=-1) * (bmax - bmin)
    return SdfVolume(dims, bmin.astype(np.float32), bmax.astype(np.float32),
                     fn(p).astype(np.float32).reshape(-1))


def sphere_sdf(center, radius):
    c = np.asarray(center, np.float64)
    return lambda p: np.linalg.norm(p - c, axis=-1) - radius


def sphere_union_ellipsoid_sdf(center, radius, e_center, e_radii):
    c = np.asarray(center, np.float64)
    ec = np.asarray(e_center, np.float64)
    er = np.asarray(e_radii, np.float64)

    def f(p):
        ds = np.linalg.norm(p - c, axis=-1) - radius
        q = (p - ec) / er
        k = np.linalg.norm(q, axis=-1)
        de = (k - 1.0) * np.min(er)  # approximate ellipsoid distance
        return np.minimum(ds, de)
    return f


def framing_camera(center, radius: float) -> Camera:
    dist = radius / math.tan(math.radians(15.0)) / 0.8
    c = np.asarray(center, np.float64)
    return Camera(eye=c + np.array([0.0, 0.0, dist]), target=c)


def sphere_depth(width: int, height: int, camera: Camera, center, radius: float) -> np.ndarray:
    """NDC depth of a sphere at texel centres; 1.0 where nothing is hit.
    Row 0 is the top of the image (texture coordinates)."""
    view = M.to_rows(camera.view())
    proj = M.to_rows(camera.proj(width, height))
    inv_vp = np.linalg.inv(proj @ view)
    xs = (np.arange(width) + 0.5) / width * 2.0 - 1.0
    ys = 1.0 - (np.arange(height) + 0.5) / height * 2.0
    X, Y = np.meshgrid(xs, ys)
    near = np.stack([X, Y, np.zeros_like(X), np.ones_like(X)], -1) @ inv_vp.T
    far = np.stack([X, Y, np.ones_like(X), np.ones_like(X)], -1) @ inv_vp.T
    o = near[..., :3] / near[..., 3:]
    dvec = _unit(far[..., :3] / far[..., 3:] - o)
    oc = o - np.asarray(center, np.float64)
    b = np.sum(oc * dvec, -1)
    cc = np.sum(oc * oc, -1) - radius * radius
    disc = b * b - cc
    t = -b - np.sqrt(np.maximum(disc, 0.0))
    hit = o + t[..., None] * dvec
    clip = np.concatenate([hit, np.ones_like(t)[..., None]], -1) @ (proj @ view).T
    z = clip[..., 2] / clip[..., 3]
    depth = np.where((disc >= 0.0) & (t > 0.0), z, 1.0)
    return depth.astype(np.float32).reshape(-1)


@dataclasses.dataclass
class Instance:
    """One hair instance of a workload: its static data and camera."""
    cfg: HairConfig
    sim: SimulationParams
    hair: HairBuffers
    sdf: SdfVolume
    scene: SceneParams
    scene_depth: np.ndarray   # mesh depth for the tiles / fine depth tests
    head_center: np.ndarray
    head_radius: float
    wind_dir: np.ndarray
    wind_amplitude: float = 0.0
    wind_frequency_hz: float = 0.5

    @property
    def width(self) -> int:
        return self.scene.width

    @property
    def height(self) -> int:
        return self.scene.height

    def wind_strength(self, frame_idx: int) -> float:
        return float(self.wind_amplitude * math.sin(
            2.0 * math.pi * self.wind_frequency_hz * frame_idx * self.sim.delta_time))


def make_instance(rng, *, strands, points, width, height, tile_size=16, depth_bins=8,
                  slices=4, shading_points=8, grid_dims=32, sdf_dims=32, iterations=7,
                  curl=False, ponytail=0.0, ellipsoid=False, wind_amplitude=0.0,
                  fiber_radius=5e-4, dt=1.0 / 60.0, processor_count=0,
                  avg_segments_per_tile=128) -> Instance:
    head_c = np.zeros(3)
    head_r = 0.1
    asset = grow_hair(rng, strands, points, center=head_c, head_radius=head_r,
                      curl=curl, ponytail_fraction=ponytail)
    hb = build_hair_buffers(asset)
    cfg = HairConfig(tile_size=tile_size, tile_depth_bins=depth_bins, slices_per_pixel=slices,
                     shading_points=shading_points, grid_dims=grid_dims,
                     processor_count=processor_count, avg_segments_per_tile=avg_segments_per_tile)
    wind_dir = _unit(rng.standard_normal(3)) if wind_amplitude else \
        M.spherical_to_cartesian(18.0, 91.0)
    sim = SimulationParams(delta_time=dt, constraint_iterations=iterations,
                           collision_sphere=(head_c[0], head_c[1], head_c[2], head_r),
                           wind_strength=0.0)
    R = float(hb.sphere_radius) * 1.1
    sdf_min = hb.sphere_center.astype(np.float64) - R
    sdf_max = hb.sphere_center.astype(np.float64) + R
    if ellipsoid:
        fn = sphere_union_ellipsoid_sdf(head_c, head_r, head_c + np.array([0.0, -0.17, 0.02]),
                                        (0.16, 0.07, 0.09))
    else:
        fn = sphere_sdf(head_c, head_r)
    sdf = sdf_from_function(fn, sdf_dims, sdf_min, sdf_max)
    gmin, gmax = scale_bounding_box(hb.bbox[0], hb.bbox[1], sim.grid_scale)
    cam = framing_camera(hb.sphere_center, float(hb.sphere_radius))
    scene = SceneParams(width=width, height=height, camera=cam, fiber_radius=fiber_radius,
                        sdf_bounds=(sdf.bounds_min, sdf.bounds_max), grid_bounds=(gmin, gmax),
                        hair_sphere=(hb.sphere_center, float(hb.sphere_radius)),
                        collision_sphere=sim.collision_sphere,
                        sdf_distance_offset=sim.sdf_distance_offset)
    depth = sphere_depth(width, height, cam, head_c, head_r * 0.98)
    return Instance(cfg, sim, hb, sdf, scene, depth, head_c, head_r, np.asarray(wind_dir),
                    wind_amplitude=wind_amplitude)


def sdf_depth(width: int, height: int, camera: Camera, vol: SdfVolume, scale: int = 4,
              steps: int = 96) -> np.ndarray:
    """NDC depth of the SDF's zero surface seen by the camera (sphere tracing
    on the host, trilinear distances, at 1/scale of the viewport then
    repeated to it); 1.0 where a ray misses.  Row 0 is the top."""
    w, h = max(1, width // scale), max(1, height // scale)
    view = M.to_rows(camera.view())
    proj = M.to_rows(camera.proj(width, height))
    vp = proj @ view
    inv_vp = np.linalg.inv(vp)
    xs = (np.arange(w) + 0.5) / w * 2.0 - 1.0
    ys = 1.0 - (np.arange(h) + 0.5) / h * 2.0
    X, Y = np.meshgrid(xs, ys)
    near = np.stack([X, Y, np.zeros_like(X), np.ones_like(X)], -1) @ inv_vp.T
    far = np.stack([X, Y, np.ones_like(X), np.ones_like(X)], -1) @ inv_vp.T
    o = (near[..., :3] / near[..., 3:]).reshape(-1, 3)
    d = _unit(far[..., :3] / far[..., 3:] - near[..., :3] / near[..., 3:]).reshape(-1, 3)
    D = vol.dims
    lo, hi = np.asarray(vol.bounds_min, np.float64), np.asarray(vol.bounds_max, np.float64)
    grid = vol.distances.reshape(D, D, D).astype(np.float64)  # [z][y][x]

    def dist(p):
        t = np.clip((p - lo) / (hi - lo), 0.0, 1.0) * D - 0.5
        i0 = np.clip(np.floor(t).astype(np.int64), 0, D - 1)
        i1 = np.clip(i0 + 1, 0, D - 1)
        f = np.clip(t - np.floor(t), 0.0, 1.0)
        out = 0.0
        for dz in (0, 1):
            for dy in (0, 1):
                for dx in (0, 1):
                    wgt = ((f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1])
                           * (f[:, 2] if dz else 1 - f[:, 2]))
                    out = out + wgt * grid[(i1 if dz else i0)[:, 2], (i1 if dy else i0)[:, 1], (i1 if dx else i0)[:, 0]]
        # outside the volume the distance grows at least with the distance to it
        outside = np.linalg.norm(p - np.clip(p, lo, hi), axis=1)
        return out + outside

    # start where the ray enters the volume's box
    with np.errstate(divide="ignore", invalid="ignore"):
        t0 = (lo - o) / d
        t1 = (hi - o) / d
    tmin = np.nanmax(np.minimum(t0, t1), axis=1).clip(0.0)
    tmax = np.nanmin(np.maximum(t0, t1), axis=1)
    t = tmin.copy()
    hit = np.zeros(len(o), bool)
    alive = tmax > tmin
    eps = float(np.min(hi - lo)) * 1e-3
    for _ in range(steps):
        if not alive.any():
            break
        idx = np.nonzero(alive)[0]
        dd = dist(o[idx] + t[idx, None] * d[idx])
        h_now = dd < eps
        hit[idx[h_now]] = True
        t[idx] += np.maximum(dd, eps * 0.5)
        alive[idx[h_now | (t[idx] > tmax[idx])]] = False
    p = o + t[:, None] * d
    clip = np.concatenate([p, np.ones((len(p), 1))], -1) @ vp.T
    z = np.where(hit, clip[:, 2] / clip[:, 3], 1.0).reshape(h, w)
    z = np.repeat(np.repeat(z, scale, 0), scale, 1)
    full = np.ones((height, width))
    full[: z.shape[0], : z.shape[1]] = z[:height, :width]
    return full.astype(np.float32).reshape(-1)


def asset_instance(tfx: bytes, sdf: bytes | None = None, width: int = 1920, height: int = 1080,
                   **cfg_kw) -> Instance:
    """A hair asset in the reference's file formats (a TFX file and,
    optionally, the binary SDF of its head), set up as the reference's
    default scene: CONFIG's pass constants (tile 8, 32 depth bins, 8 slices,
    64 shading points, 64^3 grids, 7 iterations) unless given, its
    simulation settings and collision sphere (constants.ts:186-340), the
    camera framing the hair's bounding sphere.  The scene depth is the SDF's
    zero surface (the head) where an SDF is given, else the collision
    sphere's."""
    from .formats import parse_sdf, parse_tfx
    asset = parse_tfx(tfx)
    hb = build_hair_buffers(asset)
    cfg = HairConfig(**cfg_kw)
    sim = SimulationParams()
    if sdf is not None:
        vol = parse_sdf(sdf)
    else:
        R = float(hb.sphere_radius) * 1.1
        c = hb.sphere_center.astype(np.float64)
        cs = sim.collision_sphere
        vol = sdf_from_function(sphere_sdf(np.asarray(cs[:3]), cs[3]), 32, c - R, c + R)
    gmin, gmax = scale_bounding_box(hb.bbox[0], hb.bbox[1], sim.grid_scale)
    cam = framing_camera(hb.sphere_center, float(hb.sphere_radius))
    scene = SceneParams(width=width, height=height, camera=cam,
                        sdf_bounds=(vol.bounds_min, vol.bounds_max), grid_bounds=(gmin, gmax),
                        hair_sphere=(hb.sphere_center, float(hb.sphere_radius)),
                        collision_sphere=sim.collision_sphere, sdf_distance_offset=sim.sdf_distance_offset)
    cs = np.asarray(sim.collision_sphere[:3], np.float64)
    depth = sdf_depth(width, height, cam, vol) if sdf is not None else \
        sphere_depth(width, height, cam, cs, sim.collision_sphere[3])
    return Instance(cfg, sim, hb, vol, scene, depth, cs, float(sim.collision_sphere[3]),
                    np.asarray(M.spherical_to_cartesian(sim.wind_dir_phi, sim.wind_dir_theta)))


def plain_small(seed: int = 0, **kw) -> Instance:
    """2,000 x 16 strands at 640x480, tiles 16, 8 bins, 4 slices, 8 shading
    points, 32^3 sphere SDF and grids, one step at dt 1/60, no wind."""
    rng = np.random.Generator(np.random.PCG64(seed))
    args = dict(strands=2000, points=16, width=640, height=480, depth_bins=8, slices=4,
                shading_points=8)
    args.update(kw)
    return make_instance(rng, **args)


def plain_full(seed: int = 0, **kw) -> Instance:
    """10,000 x 32 curly strands at 1920x1080, 16 bins, 4 slices, 16 shading
    points, 4 iterations, 64^3 sphere-union-ellipsoid SDF, random wind
    direction with sinusoidal strength of amplitude 1.

    Grids are 64^3 (the reference's default): at 32^3 this density of
    strands overflows the reference's i32 fixed-point density grid (x1e6,
    wrapping atomics) near the roots on the very first splat, and the
    simulation blows strands apart within a few frames -- on the reference's
    arithmetic as on this one.  ``grid_dims=32`` reproduces that."""
    rng = np.random.Generator(np.random.PCG64(seed))
    args = dict(strands=10000, points=32, width=1920, height=1080, depth_bins=16, slices=4,
                shading_points=16, iterations=4, sdf_dims=64, grid_dims=64, curl=True, ellipsoid=True,
                wind_amplitude=1.0)
    args.update(kw)
    return make_instance(rng, **args)


def stress(seed: int = 0, **kw) -> Instance:
    """200,000 x 32 strands, 60% in a ponytail cone, 3840x2160, 32 bins,
    8 slices, 32 shading points, 128^3 SDF, 64^3 grids, 8 iterations."""
    rng = np.random.Generator(np.random.PCG64(seed))
    args = dict(strands=200000, points=32, width=3840, height=2160, depth_bins=32, slices=8,
                shading_points=32, iterations=8, sdf_dims=128, grid_dims=64, ponytail=0.6,
                ellipsoid=True, avg_segments_per_tile=1024)
    args.update(kw)
    return make_instance(rng, **args)


def batched_instances(seed: int = 0, count: int = 64, tile_size=16, depth_bins=8, **kw):
    """64 instances: strands U[1k, 20k], points in {16, 24, 32}, square
    resolution in {256, 512, 1024}, own camera and own 32^3 SDF each."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        s = int(rng.integers(1000, 20001))
        p = int(rng.choice([16, 24, 32]))
        r = int(rng.choice([256, 512, 1024]))
        out.append(make_instance(rng, strands=s, points=p, width=r, height=r,
                                 tile_size=tile_size, depth_bins=depth_bins, **kw))
    return out
