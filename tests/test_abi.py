"""The C-ABI library loads and exports exactly what include/charm_gpu.h declares (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np

from charm_3d_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions() -> list[str]:
    src = open(os.path.join(ROOT, "include", "charm_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(charm_(?:gpu|host)_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "charm_gpu_step" in names and "charm_gpu_upload_mesh" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = abi.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    bound = {n for n, _, _ in abi.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_struct_sizes_match_binding():
    lib = abi.load()
    out = np.zeros(6, np.int64)
    assert lib.charm_gpu_abi_sizes(out.ctypes.data_as(C.POINTER(C.c_int64))) == 0
    assert out[0] == C.sizeof(abi.Config)
    assert out[1] == C.sizeof(abi.Mesh)
    assert out[2] == C.sizeof(abi.Comp)
    assert out[3] == C.sizeof(abi.Bnd)
    assert out[4] == C.sizeof(abi.Objective)
    assert out[5] == C.sizeof(abi.AdjointInfo)


def test_version_string():
    assert b"sm_103a" in abi.load().charm_gpu_version()
