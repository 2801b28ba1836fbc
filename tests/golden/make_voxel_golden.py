"""Golden voxel flags from the reference itself: runs oracle/_ref/plb_voxel
(the reference's voxelize(mesh, domain, borderWidth) on a TriangleSet built
from the triangles) on every mesh of voxcases.py for border widths 0-2, and on
the edge-touch box, and writes tests/golden/voxel_reference.npz (triangles,
box, width and flags of each case).

    make -f oracle/Makefile.ref REF=<reference>   # builds oracle/_ref/plb_voxel
    python tests/golden/make_voxel_golden.py
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "plb_voxel")
sys.path[:0] = [ROOT, HERE]

import voxcases  # noqa: E402
from palabos_gb300 import meshes  # noqa: E402


def reference_voxelize(tri, shape, width, tmp):
    tri = np.ascontiguousarray(tri, np.float64).reshape(-1, 9)
    c, r = os.path.join(tmp, "case"), os.path.join(tmp, "result")
    with open(c, "wb") as f:
        f.write(b"PLBVOX01" + struct.pack("<5i", *shape, width, tri.shape[0]) + tri.tobytes())
    subprocess.run([DRIVER, c, r], check=True, stdout=subprocess.DEVNULL)
    with open(r, "rb") as f:
        data = f.read()
    assert data[:8] == b"PLBVXR01" and struct.unpack_from("<3i", data, 8) == tuple(shape)
    return np.frombuffer(data, "<i4", offset=20).reshape(shape).astype(np.int8)


def main():
    if not os.path.exists(DRIVER):
        raise SystemExit("build oracle/_ref/plb_voxel first (make -f oracle/Makefile.ref)")
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name in sorted(voxcases.CASES):
            make, shape = voxcases.CASES[name]
            tri = make()
            out[f"{name}__tri"] = tri
            out[f"{name}__shape"] = np.array(shape)
            for w in voxcases.WIDTHS:
                out[f"{name}__w{w}"] = reference_voxelize(tri, shape, w, tmp)
        lo, hi, seg, shape = voxcases.EDGE_TOUCH
        tri = meshes.cuboid(lo, hi, seg)
        out["edge_touch__tri"] = tri
        out["edge_touch__shape"] = np.array(shape)
        out["edge_touch__w1"] = reference_voxelize(tri, shape, 1, tmp)
    np.savez_compressed(os.path.join(HERE, "voxel_reference.npz"), **out)
    print(f"{len(voxcases.CASES)} meshes x {len(voxcases.WIDTHS)} widths + the edge-touch box")


if __name__ == "__main__":
    main()
