// Double-word arithmetic on the FP32 pipe: a value is an unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi)/2, about 48 significant bits.
// GB300 issues FP32 at 64x its FP64 rate, so the flux arithmetic of the DW
// form (CHARM_GPU_PREC_DW) runs in this type: each operation costs a few
// FP32 instructions instead of one FP64 instruction, and lands within a few
// units of 2^-48 relative of the exact result.
//
// The algorithms are the published error-free transformations and
// double-word operations: TwoSum (Knuth, TAOCP vol. 2), Fast2Sum (Dekker,
// 1971), TwoProd by a fused multiply-add, and the double-word sum, product,
// quotient and square root of M. Joldes, J.-M. Muller, V. Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word
// arithmetic", ACM TOMS 44(2), 2017 (AccurateDWPlusDW, DWTimesDW with FMA,
// Dekker-style division and square root with one correction step).
//
// Exponent range is the float range: the flux arithmetic of this solver
// stays within it (states ~1e-3..1e7); values below ~1e-30 lose low bits in
// lo.  exp and log go through FP64 (they appear only off the ideal-gas path).
#pragma once

#include <cmath>

namespace charm {

// The overloads below for dw would hide the global float and double ones
// from unqualified calls inside this namespace; bring those in beside them.
using ::sqrt;
using ::fabs;
using ::fmax;
using ::fmin;
using ::exp;
using ::log;
using ::isfinite;

struct dw {
    float h, l;

    dw() = default;
    __host__ __device__ constexpr dw(float hi, float lo) : h(hi), l(lo) {}
    // from a double: hi the rounding of d, lo the rounding of the remainder
    // (folded at compile time for constants)
    __host__ __device__ constexpr dw(double d) : h((float) d), l((float) (d - (double) (float) d)) {}
    __host__ __device__ constexpr dw(float f) : h(f), l(0.f) {}
    __host__ __device__ constexpr dw(int i) : h((float) i), l(0.f) {}
    __host__ __device__ explicit operator double() const { return (double) h + (double) l; }
};

// ---- error-free transformations ---------------------------------------------

__device__ __forceinline__ dw dw_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return dw(s, e);
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ dw dw_fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return dw(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dw dw_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return dw(p, __fmaf_rn(a, b, -p));
}

// ---- arithmetic ---------------------------------------------------------------

__device__ __forceinline__ dw operator+(dw x, dw y)
{
    dw s = dw_two_sum(x.h, y.h);
    const dw t = dw_two_sum(x.l, y.l);
    s = dw_fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return dw_fast_two_sum(s.h, __fadd_rn(s.l, t.l));
}

__device__ __forceinline__ dw operator-(dw x) { return dw(-x.h, -x.l); }
__device__ __forceinline__ dw operator-(dw x, dw y) { return x + (-y); }

__device__ __forceinline__ dw operator*(dw x, dw y)
{
    const dw c = dw_two_prod(x.h, y.h);
    const float t = __fmaf_rn(x.h, y.l, __fmul_rn(x.l, y.h));
    return dw_fast_two_sum(c.h, __fadd_rn(c.l, t));
}

// x * f for a float f (one product less)
__device__ __forceinline__ dw dw_mul_f(dw x, float f)
{
    const dw c = dw_two_prod(x.h, f);
    return dw_fast_two_sum(c.h, __fmaf_rn(x.l, f, c.l));
}

// Dekker's quotient with one correction: q1 = xh / yh, r = x - y q1,
// q = q1 + rh / yh
__device__ __forceinline__ dw operator/(dw x, dw y)
{
    const float q1 = __fdiv_rn(x.h, y.h);
    const dw r = x - dw_mul_f(y, q1);
    return dw_fast_two_sum(q1, __fdiv_rn(r.h, y.h));
}

__device__ __forceinline__ dw &operator+=(dw &x, dw y) { return x = x + y; }
__device__ __forceinline__ dw &operator-=(dw &x, dw y) { return x = x - y; }
__device__ __forceinline__ dw &operator*=(dw &x, dw y) { return x = x * y; }

// ---- comparisons (hi first, lo breaks ties) ----------------------------------

__device__ __forceinline__ bool operator<(dw x, dw y) { return x.h < y.h || (x.h == y.h && x.l < y.l); }
__device__ __forceinline__ bool operator>(dw x, dw y) { return y < x; }
__device__ __forceinline__ bool operator<=(dw x, dw y) { return x.h < y.h || (x.h == y.h && x.l <= y.l); }
__device__ __forceinline__ bool operator>=(dw x, dw y) { return y <= x; }
__device__ __forceinline__ bool operator==(dw x, dw y) { return x.h == y.h && x.l == y.l; }
__device__ __forceinline__ bool operator!=(dw x, dw y) { return !(x == y); }

// ---- functions ------------------------------------------------------------------

__device__ __forceinline__ dw fabs(dw x) { return (x.h < 0.f || (x.h == 0.f && x.l < 0.f)) ? -x : x; }
__device__ __forceinline__ dw fmax(dw x, dw y) { return (x < y) ? y : x; }
__device__ __forceinline__ dw fmin(dw x, dw y) { return (y < x) ? y : x; }
__device__ __forceinline__ bool isfinite(dw x) { return ::isfinite(x.h) && ::isfinite(x.l); }

// s = sqrt(hi); x - s^2 exactly to first order; s + (x - s^2) / (2 s)
__device__ __forceinline__ dw sqrt(dw x)
{
    if (!(x.h > 0.f)) return dw(sqrtf(x.h), 0.f);   // 0 -> 0, negative -> NaN
    const float s = __fsqrt_rn(x.h);
    const dw p = dw_two_prod(s, s);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(x.h, p.h), p.l), x.l);
    return dw_fast_two_sum(s, __fdiv_rn(r, __fmul_rn(2.f, s)));
}

__device__ __forceinline__ dw exp(dw x) { return dw(::exp((double) x)); }
__device__ __forceinline__ dw log(dw x) { return dw(::log((double) x)); }

}  // namespace charm
