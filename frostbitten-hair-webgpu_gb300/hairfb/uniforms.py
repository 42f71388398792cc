"""Byte-exact packers for the two uniform blocks the hair passes consume.

- ``Uniforms`` (1184 B): RenderUniformsBuffer, struct at
  src/passes/renderUniformsBuffer.ts:105-137, packer ``update()`` at :205-288.
- ``SimulationUniforms`` (304 B): SimulationUniformsBuffer, struct at
  src/passes/simulation/simulationUniformsBuffer.ts:19-51, packer at :86-152.

The CUDA library and the oracle both read these raw bytes, exactly as the
WGSL passes read the uniform buffers the reference uploads with
``queue.writeBuffer`` (src/utils/typedArrayView.ts:70-78).
"""
from __future__ import annotations

import dataclasses
import math
import struct

import numpy as np

from . import matrices as M
from .config import HairConfig, SimulationParams

RENDER_UNIFORMS_BYTES = 1184
SIM_UNIFORMS_BYTES = 304

# Uniforms byte offsets (WGSL layout rules, renderUniformsBuffer.ts:105-137)
OFF = dict(
    vpMatrix=0, vpMatrixInv=64, viewMatrix=128, projMatrix=192, projMatrixInv=256,
    modelMatrix=320, modelViewMat=384, mvpMatrix=448, collisionSphereModelMatrix=512,
    viewport=576, cameraPosition=592, colorMgmt=608, lightAmbient=624,
    light0=640, light1=672, light2=704, shadows=736, ao=960, hairMaterial=992,
    sdf=1056, gridData=1088, fiberRadius=1120, dbgShadowMapPreviewSize=1124,
    maxDrawnHairSegments=1128, displayMode=1132, background=1136,
    collisionSpherePosition=1168, gizmoActiveState=1180,
)

SIM_OFF = dict(
    modelMatrix=0, modelMatrixInv=64, collisionSphere=128, wind=144, sdf=160,
    gridData=192, deltaTime=224, gravity=228, constraintIterations=232, frameIdx=236,
    windStrengthLull=240, windColisionTraceOffset=244, stiffnessLengthConstr=248,
    stiffnessCollisions=252, stiffnessSDF=256, volumePreservation=260, friction=264,
    stiffnessGlobalConstr=268, globalConstrExtent=272, globalConstrFade=276,
    stiffnessLocalConstr=280, windPhaseOffset=284, windStrengthFrequency=288,
    windStrengthJitter=292,
)

DISPLAY_MODE_FINAL = 0
DISPLAY_MODE_USED_SLICES = 4


def _col(*rgb):
    """col(), src/constants.ts:370-376: 0-255 -> 0-1."""
    return tuple(c / 255.0 for c in rgb)


@dataclasses.dataclass
class Light:
    phi: float
    theta: float
    color: tuple
    energy: float


@dataclasses.dataclass
class HairMaterial:
    """CONFIG.hairRender.material, src/constants.ts:203-215"""
    color0: tuple = _col(119, 43, 119)
    color1: tuple = _col(76, 0, 255)
    specular: float = 0.9
    weight_tt: float = 0.0
    weight_trt: float = 1.4
    shift: float = 0.0
    roughness: float = 0.3
    color_rng: float = 0.1
    luma_rng: float = 0.1
    attenuation: float = 30.0
    shadows: float = 0.5


def default_lights():
    """CONFIG.lights, src/constants.ts:146-151"""
    return [Light(60.0, 20.0, _col(255, 244, 204), 0.8),
            Light(100.0, 97.0, _col(204, 249, 255), 0.8),
            Light(-90.0, 30.0, _col(255, 242, 204), 0.8)]


class _Writer:
    """TypedArrayView-like sequential writer (src/utils/typedArrayView.ts)."""

    def __init__(self, size: int):
        self.buf = bytearray(size)
        self.off = 0

    def f32(self, v):
        struct.pack_into("<f", self.buf, self.off, float(v))
        self.off += 4

    def u32(self, v):
        struct.pack_into("<I", self.buf, self.off, int(math.floor(v)) & 0xFFFFFFFF)
        self.off += 4

    def mat4(self, m):
        for x in np.asarray(m, dtype=np.float32).reshape(16):
            self.f32(x)

    def seek(self, off: int):
        self.off = off


@dataclasses.dataclass
class Camera:
    """Per-instance camera: matrices the host builds for the passes."""
    eye: np.ndarray
    target: np.ndarray
    fov_deg: float = 30.0
    near: float = 0.01
    far: float = 100.0

    def view(self) -> np.ndarray:
        return M.look_at(self.eye, self.target)

    def proj(self, width: int, height: int) -> np.ndarray:
        """createCameraProjectionMat, src/utils/matrices.ts:5-16"""
        return M.perspective(math.radians(self.fov_deg), width / height, self.near, self.far)


@dataclasses.dataclass
class SceneParams:
    """Everything the render-uniform packer needs for one instance."""
    width: int
    height: int
    camera: Camera
    fiber_radius: float = 0.0006
    model_matrix: np.ndarray = dataclasses.field(default_factory=M.identity)
    material: HairMaterial = dataclasses.field(default_factory=HairMaterial)
    lights: list = dataclasses.field(default_factory=default_lights)
    light_ambient: tuple = (1.0, 1.0, 1.0, 0.05)
    sdf_bounds: tuple = ((0, 0, 0), (1, 1, 1))
    grid_bounds: tuple = ((0, 0, 0), (1, 1, 1))
    hair_sphere: tuple = ((0.0, 0.0, 0.0), 1.0)
    collision_sphere: tuple = (-0.18, 1.56, 0.06, 0.06)
    sdf_distance_offset: float = -0.0015
    display_mode: int = DISPLAY_MODE_FINAL
    display_mode_extra: int = 0
    # shadows (CONFIG.shadows, constants.ts:154-176)
    shadow_source_phi: float = 37.0
    shadow_source_theta: float = 45.0
    shadow_source_distance: float = 5.0
    shadow_target: tuple = (0.0, 2.0, 0.0)
    use_pcss: bool = False
    pcf_radius: int = 3
    shadow_bias: float = 0.0005
    shadow_strength: float = 0.4
    ao_strength: float = 0.4


def shadow_source_matrices(p: SceneParams):
    """getShadowSource{WorldPosition,ViewMatrix,ProjectionMatrix},
    src/passes/shadowMapPass/shared/getMVP_ShadowSourceMatrix.ts:14-73"""
    pos = M.spherical_to_cartesian(p.shadow_source_phi, p.shadow_source_theta) * p.shadow_source_distance
    target = M.transform_point(p.model_matrix, p.shadow_target)[:3]
    view = M.look_at(pos, target)
    mv = M.multiply(view, p.model_matrix)
    c, r = p.hair_sphere
    sp = M.transform_point(mv, c)
    m = 1.05
    proj = M.ortho((sp[0] - r) * m, (sp[0] + r) * m, (sp[1] - r) * m, (sp[1] + r) * m, 0.1, 20.0)
    return pos, view, proj


def pack_render_uniforms(p: SceneParams, cfg: HairConfig, max_drawn: int | None = None) -> bytes:
    """RenderUniformsBuffer.update(), renderUniformsBuffer.ts:205-288."""
    view = p.camera.view()
    proj = p.camera.proj(p.width, p.height)
    vp = M.multiply(proj, view)
    model = np.asarray(p.model_matrix, dtype=np.float32)
    w = _Writer(RENDER_UNIFORMS_BYTES)
    w.mat4(vp)
    w.mat4(M.invert(vp))
    w.mat4(view)
    w.mat4(proj)
    w.mat4(M.invert(proj))
    w.mat4(model)
    w.mat4(M.multiply(view, model))
    w.mat4(M.multiply(proj, M.multiply(view, model)))
    cs = p.collision_sphere
    r = cs[3] * 0.95
    w.mat4(M.scale(M.translation(cs[:3]), (r, r, r)))
    # viewport, camera position, color mgmt, ambient
    for v in (p.width, p.height, 0.0, 0.0):
        w.f32(v)
    for v in (*np.asarray(p.camera.eye, dtype=np.float64)[:3], 0.0):
        w.f32(v)
    for v in (2.2, 0.85, 1.0, 0.0):
        w.f32(v)
    for v in p.light_ambient:
        w.f32(v)
    for light in p.lights:  # writeLight, :290-306
        pos = M.spherical_to_cartesian(light.phi, light.theta) * 2.0
        for v in (*pos, 0.0, *light.color, light.energy):
            w.f32(v)
    # writeShadows, :308-343
    spos, sview, sproj = shadow_source_matrices(p)
    w.mat4(M.multiply(sview, model))
    w.mat4(sproj)
    w.mat4(M.multiply(sproj, M.multiply(sview, model)))
    for v in (*spos, p.fiber_radius):
        w.f32(v)
    w.u32(1 if p.use_pcss else 0)
    w.u32(p.pcf_radius)
    w.f32(p.shadow_bias)
    w.f32(p.shadow_strength)
    # writeAo, :345-358 (CONFIG.ao)
    for v in (2.0, 0.0, 0.16, 4.0):
        w.f32(v)
    w.u32(12)
    w.u32(8)
    w.f32(p.ao_strength)
    w.u32(0)
    # writeHairMaterial, :360-382
    m = p.material
    for v in (*m.color0, m.specular, *m.color1, m.shadows, m.weight_tt, m.weight_trt,
              m.shift, m.roughness, m.color_rng, m.luma_rng, m.attenuation, 0.0):
        w.f32(v)
    # SDFCollider.writeToDataView, sdfCollider.ts:77-91
    smin, smax = p.sdf_bounds
    for v in (*smin, 0.5 + 2.0, *smax, p.sdf_distance_offset):
        w.f32(v)
    # GridData.writeToDataView, gridData.ts:93-106
    gmin, gmax = p.grid_bounds
    for v in (*gmin, 0.5, *gmax):
        w.f32(v)
    w.u32(1 + 16)
    # misc
    w.f32(p.fiber_radius)
    w.f32(0.0)
    w.u32(cfg.max_drawn_segments(p.width, p.height) if max_drawn is None else max_drawn)
    w.u32(p.display_mode | (p.display_mode_extra << 8))
    # background (CONFIG.background)
    for v in (*_col(22, 162, 188), 5.0, *_col(14, 103, 120), 0.5):
        w.f32(v)
    for v in cs[:3]:
        w.f32(v)
    w.u32(3)
    assert w.off == RENDER_UNIFORMS_BYTES
    return bytes(w.buf)


def pack_sim_uniforms(sim: SimulationParams, model_matrix, sdf_bounds, grid_bounds,
                      frame_idx: int, wind_dir=None, wind_strength=None) -> bytes:
    """SimulationUniformsBuffer.update(), simulationUniformsBuffer.ts:86-152."""
    model = np.asarray(model_matrix, dtype=np.float32)
    inv = M.invert(model)
    w = _Writer(SIM_UNIFORMS_BYTES)
    w.mat4(model)
    w.mat4(inv)
    cs = sim.collision_sphere
    os_ = M.to_rows(inv) @ np.array([cs[0], cs[1], cs[2], 1.0])
    for v in (os_[0], os_[1], os_[2], cs[3]):
        w.f32(v)
    if wind_dir is None:
        wind_dir = M.spherical_to_cartesian(sim.wind_dir_phi, sim.wind_dir_theta)
    wd = M.to_rows(inv) @ np.array([wind_dir[0], wind_dir[1], wind_dir[2], 0.0])
    for v in (wd[0], wd[1], wd[2], sim.wind_strength if wind_strength is None else wind_strength):
        w.f32(v)
    smin, smax = sdf_bounds
    for v in (*smin, 0.5 + 2.0, *smax, sim.sdf_distance_offset):
        w.f32(v)
    gmin, gmax = grid_bounds
    for v in (*gmin, 0.5, *gmax):
        w.f32(v)
    w.u32(1 + 16)
    w.f32(sim.delta_time)
    w.f32(sim.gravity)
    w.u32(sim.constraint_iterations)
    w.u32(frame_idx)
    for v in (sim.wind_strength_lull, sim.wind_collision_trace_offset, sim.stiffness_length,
              sim.stiffness_collisions, sim.stiffness_sdf, sim.volume_preservation, sim.friction,
              sim.stiffness_global, sim.global_extent, sim.global_fade, sim.stiffness_local,
              sim.wind_phase_offset, sim.wind_strength_frequency, sim.wind_strength_jitter,
              0.0, 0.0):
        w.f32(v)
    assert w.off == SIM_UNIFORMS_BYTES
    return bytes(w.buf)


# Byte offsets of the two fields of SimulationUniforms that change from frame
# to frame when the scene does not (simulationUniformsBuffer.ts:19-51): the
# wind strength (.w of the wind vector) and frameIdx.
SIM_WIND_STRENGTH_OFFSET = 156
SIM_FRAME_IDX_OFFSET = 236


def patch_sim_uniforms(block: bytearray, frame_idx: int, wind_strength: float) -> None:
    """Rewrites frameIdx and the wind strength of a packed SimulationUniforms
    block in place: the same bytes as pack_sim_uniforms for that frame."""
    struct.pack_into("<f", block, SIM_WIND_STRENGTH_OFFSET, float(wind_strength))
    struct.pack_into("<I", block, SIM_FRAME_IDX_OFFSET, int(math.floor(frame_idx)) & 0xFFFFFFFF)


def read_f32(block: bytes, off: int, n: int = 1) -> np.ndarray:
    return np.frombuffer(block, dtype=np.float32, count=n, offset=off)
