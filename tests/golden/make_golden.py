"""Regenerate the golden fixtures from the reference's own test data.

The reference pins three things with binary fixtures next to its tests:

- src/passes/swHair/__test__/swRasterizer.snapshot.bin -- 128x128 u32 ABGR
  output of the sw-raster utility test (swRasterizer.test.ts:57-144); stored
  here sparsely as ``swRasterizer.snapshot.npz`` (indices + values of the
  non-zero pixels, plus the shape), which is lossless.
- src/scene/sdfCollider/__test__/test-sdf.bin -- a 5^3 SDF binary
  (createSdfColliderFromBinary.test.ts:14-57), copied verbatim.
- src/scene/sdfCollider/__test__/sdf-binary.snapshot.bin -- that test's
  snapshot (each distance truncated to a u8 by the snapshot helper), copied.

Run from the repository root:  python tests/golden/make_golden.py REF_ROOT
(REF_ROOT: a checkout of the reference project)
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root: str) -> None:
    snap = os.path.join(ref_root, "src/passes/swHair/__test__/swRasterizer.snapshot.bin")
    a = np.fromfile(snap, dtype="<u4")
    nz = np.nonzero(a)[0]
    np.savez_compressed(os.path.join(HERE, "swRasterizer.snapshot.npz"),
                        size=np.array([128, 128], np.uint32), index=nz.astype(np.uint32),
                        value=a[nz].astype(np.uint32))
    for name in ("test-sdf.bin", "sdf-binary.snapshot.bin"):
        shutil.copyfile(os.path.join(ref_root, "src/scene/sdfCollider/__test__", name),
                        os.path.join(HERE, name))
    print(f"snapshot: {nz.size} lit pixels of {a.size}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REF_ROOT  (a checkout of the reference project)")
    main(sys.argv[1])
