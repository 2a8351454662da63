"""Build the test-only host library tests/native/_build/libadjoint_point.so."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def build() -> str:
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libadjoint_point.so")
    src = os.path.join(HERE, "adjoint_point.cpp")
    hdr = os.path.join(ROOT, "charm_3d_gb300", "csrc", "adjoint_math.h")
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-I" + os.path.join(ROOT, "charm_3d_gb300", "csrc"), src, "-o", out]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + res.stderr)
    return out
