"""Shared setup for the parity tests: seeded workloads run through the CUDA
library (via the C-ABI) and through the CPU oracle on the same inputs."""
from __future__ import annotations

import dataclasses

import numpy as np

from hairfb import synthetic, uniforms as UN

INVALID = 0xFFFFFFFF


def small_instance(seed=0, **kw):
    """The 2,000 x 16 workload, optionally cut down / re-tiled."""
    args = dict(strands=2000, points=16, width=640, height=480, depth_bins=8, slices=4, shading_points=8)
    args.update(kw)
    rng = np.random.Generator(np.random.PCG64(seed))
    return synthetic.make_instance(rng, **args)


@dataclasses.dataclass
class Frame:
    inst: synthetic.Instance
    uniforms: bytes
    max_drawn: int

    @property
    def cfg(self):
        return self.inst.cfg


def frame_of(inst) -> Frame:
    u = UN.pack_render_uniforms(inst.scene, inst.cfg)
    return Frame(inst, u, inst.cfg.max_drawn_segments(inst.width, inst.height))


def walk_lists(tiles, segs, max_drawn):
    """{tileBin: [encoded segments in list order]} for every non-empty head."""
    out = {}
    heads = tiles[:, 2]
    for tb in np.nonzero(heads)[0]:
        ptr = int(heads[tb]) - 1
        seq = []
        while ptr != INVALID and ptr < max_drawn:
            seq.append(int(segs[1 + 2 * ptr]))
            ptr = int(segs[2 + 2 * ptr])
            if len(seq) > max_drawn:
                raise AssertionError("cycle in a segment list")
        out[int(tb)] = seq
    return out
