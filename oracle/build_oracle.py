"""Recipe: build the CPU restatement oracle/charm_oracle.c into oracle/_build/liboracle.so.

Test infrastructure.  Builds on x86 and Arm alike (gcc, -O2,
-ffp-contract=off so both give the same bits).  Outputs are git-ignored.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
SRC = os.path.join(HERE, "charm_oracle.c")


def build(force: bool = False) -> str:
    hdr = os.path.join(ROOT, "include", "charm_gpu.h")
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr), os.path.getmtime(__file__)):
            return LIB
    os.makedirs(OUT, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-I" + os.path.join(ROOT, "include"),
           SRC, "-o", tmp, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
