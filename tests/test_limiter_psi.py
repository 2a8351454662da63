"""The Barth-Jespersen scaling from two quotients per variable equals the
reference's per-vertex minimum (CPU, IEEE arithmetic of numpy): the same
value everywhere, the same bits except the sign of a zero psi.

The reference (src/limiters/charm_limiter_bj.c:275-299) takes, over the
vertices with |df_k| > eps, min(1, (umax - u0) / df_k) for df_k > 0 and
min(1, (umin - u0) / df_k) for df_k < 0, and the minimum of those.  The
kernels (bj_side_psi in dg_device.cuh, and the FP32 form of the mixed
limiter) divide once by the largest df_k and once by the most negative:
with umax - u0 >= 0 and umin - u0 <= 0 each quotient is monotone in df_k,
and so is its correctly rounded value.  Where both bounds equal u0 the
reference's psi is -0 or +0 by which vertex comes first (0 / df_k takes
df_k's sign) and the two-quotient form gives +0: a zero either way, and
the limited coefficients psi * c are zeros either way.
"""
import numpy as np

EPS = 1e-12


def psi_reference(df, lo, hi, eps=EPS):
    """Per vertex, as the reference loops (df: [..., 8])."""
    psi = np.ones(df.shape[:-1], df.dtype)
    one = df.dtype.type(1)
    for k in range(df.shape[-1]):
        d = df[..., k]
        with np.errstate(divide="ignore", invalid="ignore"):
            pos = np.minimum(one, hi / d)
            neg = np.minimum(one, lo / d)
        pt = np.where(np.abs(d) > eps, np.where(d > 0, pos, np.where(d < 0, neg, one)), one)
        psi = np.where(pt < psi, pt, psi)
    return psi


def psi_two_quotients(df, lo, hi, eps=EPS):
    """The kernels' form: the largest and the most negative difference."""
    zero, one = df.dtype.type(0), df.dtype.type(1)
    dmax = np.maximum(df.max(axis=-1), zero)
    dmin = np.minimum(df.min(axis=-1), zero)
    with np.errstate(divide="ignore", invalid="ignore"):
        p_pos = np.where(dmax > eps, np.minimum(one, hi / dmax), one)
        p_neg = np.where(dmin < -eps, np.minimum(one, lo / dmin), one)
    return np.where(p_neg < p_pos, p_neg, p_pos)


def _cases(rng, n, dtype):
    u0 = rng.normal(size=n).astype(dtype)
    slopes = rng.normal(size=(n, 3)).astype(dtype) * rng.choice([1e-14, 1e-6, 1.0, 1e3], size=(n, 1)).astype(dtype)
    signs = np.array([[(k & 1) * 2 - 1, (k & 2) - 1, ((k & 4) >> 1) - 1] for k in range(8)], dtype) * dtype(0.5)
    f = u0[:, None] + slopes @ signs.T              # the field at the 8 vertices
    df = f - u0[:, None]
    umax = u0 + np.abs(rng.normal(size=n)).astype(dtype) * rng.choice([0.0, 1e-9, 0.1, 10.0], size=n).astype(dtype)
    umin = u0 - np.abs(rng.normal(size=n)).astype(dtype) * rng.choice([0.0, 1e-9, 0.1, 10.0], size=n).astype(dtype)
    return df, umin - u0, umax - u0


def test_two_quotients_equal_the_per_vertex_minimum_fp64():
    rng = np.random.default_rng(11)
    df, lo, hi = _cases(rng, 400_000, np.float64)
    # edge cases: differences at +-eps, zero, one vertex only, bounds equal to u0
    df[:8] = 0.0
    df[8:16, 0] = EPS
    df[16:24, 3] = -EPS
    df[24:32, 5] = 2 * EPS
    hi[32:40] = 0.0
    lo[40:48] = 0.0
    a, b = psi_reference(df, lo, hi), psi_two_quotients(df, lo, hi)
    assert np.array_equal(a, b)
    differ = a.view(np.uint64) != b.view(np.uint64)
    assert (a[differ] == 0).all(), "bits differ only in the sign of a zero"
    assert (a < 1).mean() > 0.3, "the cases exercise the limiting branch"


def test_two_quotients_equal_the_per_vertex_minimum_fp32():
    rng = np.random.default_rng(12)
    df, lo, hi = _cases(rng, 400_000, np.float32)
    eps = np.float32(EPS)
    a, b = psi_reference(df, lo, hi, eps), psi_two_quotients(df, lo, hi, eps)
    assert np.array_equal(a, b)
    differ = a.view(np.uint32) != b.view(np.uint32)
    assert (a[differ] == 0).all(), "bits differ only in the sign of a zero"
