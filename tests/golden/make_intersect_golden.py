"""Generate tests/golden/intersect/trace_ref.txt from the reference itself.

Builds oracle/_ref/rt_ref_intersect: the reference's own Sphere / Plane / Box / BallPlane /
Model classes compiled from its sources by oracle/ref/Makefile, driven by
tests/cpp/intersect_sequence.inc (seeded rays through DrawObject::intersect, Basic3DObject.cpp:
135-551, Model.cpp:748-811), and stores what it prints: one record per call with every float as
its bit pattern. The model is the OBJ asset of tests/golden/obj, read from that directory.

    python tests/golden/make_intersect_golden.py     # needs the reference sources (x86 host)
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "rt_ref_intersect")
OUT = os.path.join(HERE, "intersect", "trace_ref.txt")
RAYS_PER_OBJECT = 300


def main() -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), EXE], check=True)
    trace = subprocess.run([EXE, str(RAYS_PER_OBJECT)], check=True, capture_output=True, text=True,
                           cwd=os.path.join(HERE, "obj")).stdout
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    with open(OUT, "w") as f:
        f.write(trace)
    print(f"{OUT}: {len(trace.splitlines())} lines")


if __name__ == "__main__":
    main()
