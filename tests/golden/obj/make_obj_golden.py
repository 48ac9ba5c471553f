"""Writes a small OBJ/MTL/BMP asset and what the reference's own loader builds from it.

The asset exercises the loader paths of the reference's Model (Model.cpp:14-349): quads with
v/vt/vn (split into two triangles), triangles with v//vn (no texture coordinates), usemtl parts,
materials that inherit the previous material's values (the reference never resets `mtl`),
`map_Kd` with a Windows path and another extension (read as <name>.bmp from the working
directory), a texture shared by two materials, comments and blank lines, a model away from the
origin (rescaled to extent 8). The expectations come from oracle/_ref/rt_ref_harness --obj (the
reference's Model::loadOBJ compiled from its sources) and are saved as model_ref.npz.

    python tests/golden/obj/make_obj_golden.py      # needs oracle/_ref/rt_ref_harness
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "rt_ref_harness")

OBJ = """# a house: walls (quads with texture coordinates), a roof (triangles without), a chimney
g house

v 1.0 0.0 2.0
v 3.0 0.0 2.0
v 3.0 2.0 2.0
v 1.0 2.0 2.0
v 1.0 0.0 4.5
v 3.0 0.0 4.5
v 3.0 2.0 4.5
v 1.0 2.0 4.5
v 2.0 3.2 3.25
v 2.5 2.4 3.0
v 2.8 2.4 3.0
v 2.8 3.1 3.0
v 2.5 3.1 3.0
vt 0.0 0.0
vt 1.0 0.0
vt 1.0 1.0
vt 0.0 1.0
vt 0.25 0.75
vt 2.5 -0.5
vn 0.0 0.0 -1.0
vn 0.0 0.0 1.0
vn -1.0 0.0 0.0
vn 1.0 0.0 0.0
vn 0.0 1.0 0.0
vn 0.0 -1.0 0.0
vn 0.0 0.6 -0.8
vn 0.0 0.6 0.8
vn -0.77 0.64 0.0
vn 0.77 0.64 0.0
usemtl wood
f 1/1/1 2/2/1 3/3/1 4/4/1
f 6/1/2 5/2/2 8/3/2 7/4/2
f 5/1/3 1/2/3 4/3/3 8/4/3
f 2/1/4 6/2/4 7/3/4 3/4/4
f 5/5/6 6/6/6 2/2/6 1/1/6

usemtl roof
f 4//7 3//7 9//7
f 7//8 8//8 9//8
f 8//9 4//9 9//9
f 3//10 7//10 9//10
usemtl metal
f 10/1/1 11/2/1 12/6/1
f 10/1/1 12/6/1 13/5/1
"""

MTL = """# three materials; later ones inherit what they do not set
newmtl wood
Ka 0.30 0.25 0.20
Kd 0.70 0.55 0.35
Ks 0.20 0.20 0.20
Ns 24
map_Kd C:\\assets\\textures\\wood.png

newmtl roof
Kd 0.60 0.15 0.10
Ns 64

newmtl metal
Ks 0.90 0.90 0.90
map_Kd wood.tga
"""


def bmp(w: int, h: int) -> bytes:
    """24-bit BMP, rows bottom-up (w*3 a multiple of 4, so no row padding)."""
    px = bytearray()
    for y in range(h):
        for x in range(w):
            px += bytes(((x * 16 + 8) & 0xFF, (y * 32 + 16) & 0xFF, 200 if (x // 4 + y // 2) % 2 else 90))
    info = struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0, 0, 2835, 2835, 0, 0)
    head = struct.pack("<2sIHHI", b"BM", 14 + 40 + len(px), 0, 0, 14 + 40)
    return head + info + bytes(px)


def write_asset() -> None:
    with open(os.path.join(HERE, "model.obj"), "w") as f:
        f.write(OBJ)
    with open(os.path.join(HERE, "model.mtl"), "w") as f:
        f.write(MTL)
    with open(os.path.join(HERE, "wood.bmp"), "wb") as f:
        f.write(bmp(16, 8))


def main() -> None:
    write_asset()
    if not os.path.exists(HARNESS):
        raise SystemExit(f"{HARNESS} missing: run `make -C oracle/ref`")
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "m")
        r = subprocess.run([HARNESS, "--obj", "model.obj", "model.mtl", out], cwd=HERE, capture_output=True, text=True,
                           check=True)
        info = json.loads(r.stdout)

        def ld(ext, dt):
            return np.fromfile(out + "." + ext, dt)

        arrays = {"tris": ld("tris.f32", np.float32).reshape(-1, 24), "tri_part": ld("tripart.i32", np.int32),
                  "part_mtl": ld("partmtl.i32", np.int32), "mtls": ld("mtls.f32", np.float32).reshape(-1, 16),
                  "mtl_tex": ld("mtltex.i32", np.int32), "tex_dims": ld("texdims.i32", np.int32).reshape(-1, 2),
                  "texels": ld("texels.u8", np.uint8), "bounds": ld("bounds.f32", np.float32)}
    np.savez_compressed(os.path.join(HERE, "model_ref.npz"), info=np.array(json.dumps(info)), **arrays)
    print(json.dumps(info))


if __name__ == "__main__":
    sys.exit(main())
