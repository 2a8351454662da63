"""The p2 basis contraction on the tensor cores (tcgen05.mma, BF16 operands
split in three terms each, FP32 accumulation in tensor memory) and on FP32
FMAs (charm_gpu_p2_interp), against the same contraction in FP64 numpy: the
values of 5 and 6 variables' 10 Taylor coefficients at the 27 cell Gauss
points (reference src/charm_base_func.c:139-196).  Bar: 1e-6 of the sum of
the magnitudes of the products (sum_i |c_i phi_i|, the denominator of the
standard error bound of a dot product; FP32 rounds at 6e-8)."""
import ctypes as C

import numpy as np
import pytest

from charm_3d_gb300 import abi

pytestmark = pytest.mark.gpu


def basis_at_gauss_points():
    g = np.array([-0.5 * np.sqrt(0.6), 0.0, 0.5 * np.sqrt(0.6)])
    gw = np.array([5.0, 8.0, 5.0]) / 18.0
    phi, w = [], []
    for q in range(27):
        ix, iy, iz = q % 3, (q // 3) % 3, q // 9
        x, y, z = g[ix], g[iy], g[iz]
        phi.append([1.0, x, y, z, x * x, y * y, z * z, x * y, x * z, y * z])
        w.append(gw[ix] * gw[iy] * gw[iz])
    return np.array(phi), np.array(w)


def run(method, coef, reps=1):
    lib = abi.load()
    V, _, E = coef.shape
    c = np.ascontiguousarray(coef, dtype=np.float32)
    s = np.empty(E)
    vals = np.empty((E, V, 27), np.float32)
    ms = C.c_double()
    rc = lib.charm_gpu_p2_interp(method, E, V, c.ctypes.data, s.ctypes.data, vals.ctypes.data, reps, C.byref(ms))
    assert rc == abi.OK, lib.charm_gpu_last_error()
    return s, vals, ms.value


@pytest.mark.parametrize("V", [5, 6])
@pytest.mark.parametrize("method", [0, 1])
def test_p2_contraction_matches_fp64(V, method):
    rng = np.random.default_rng(V)
    E = 300                                   # two full tiles of 128 and a partial one
    coef = rng.normal(size=(V, 10, E)) * np.array([1.0, 0.3, 0.3, 0.3] + [0.05] * 6)[None, :, None]
    coef[:, 0, :] += 2.0
    coef = coef.astype(np.float32)
    phi, w = basis_at_gauss_points()
    want = np.einsum("vie,qi->evq", coef.astype(np.float64), phi)
    s, vals, _ = run(method, coef)
    bound = 1e-6 * np.einsum("vie,qi->evq", np.abs(coef.astype(np.float64)), np.abs(phi))
    assert (np.abs(vals - want) <= bound).all(), (np.abs(vals - want) / bound).max()
    s_want = (w[None, None, :] * want ** 2).sum(axis=(1, 2))
    assert np.abs(s - s_want).max() <= 1e-6 * np.abs(s_want).max()


def test_tensor_core_and_fma_forms_agree():
    rng = np.random.default_rng(11)
    coef = (rng.normal(size=(6, 10, 1024)) + 1.0).astype(np.float32)
    s0, v0, _ = run(0, coef)
    s1, v1, _ = run(1, coef)
    phi, _ = basis_at_gauss_points()
    bound = 2e-6 * np.einsum("vie,qi->evq", np.abs(coef.astype(np.float64)), np.abs(phi))
    assert (np.abs(v1 - v0) <= bound).all()
    assert np.allclose(s1, s0, rtol=1e-6, atol=0.0)
