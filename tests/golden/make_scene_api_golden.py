"""Generate tests/golden/scene_api_ref.txt from the reference itself.

Builds oracle/_ref/rt_ref_scene_api (the reference's own Scene / Light / Camera / object
classes, compiled from its sources by oracle/ref/Makefile, driven by
tests/cpp/scene_api_sequence.inc) and stores what it prints: the return value of every call
of a fixed sequence of scene edits and the state after it, every float as its bit pattern.

    python tests/golden/make_scene_api_golden.py     # needs the reference sources (x86 host)
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "rt_ref_scene_api")
OUT = os.path.join(HERE, "scene_api_ref.txt")


def main() -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), EXE], check=True)
    trace = subprocess.run([EXE], check=True, capture_output=True, text=True).stdout
    with open(OUT, "w") as f:
        f.write(trace)
    print(f"{OUT}: {len(trace.splitlines())} lines")


if __name__ == "__main__":
    main()
