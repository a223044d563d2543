// pp_df.cuh -- double-float (float32 pair) arithmetic for the relaxation kernel.
//
// GB300 issues float64 at 1/64 of its float32 rate, so float64-accurate quantities of the
// FIRE loop (probe position, grid coordinate, trilinear interpolation, springs, force sum)
// are carried as unevaluated sums hi + lo of two floats (about 48 significant bits) built
// from the error-free transformations of Knuth (TwoSum), Dekker (FastTwoSum) and the
// FMA-based TwoProduct (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26 (2005)).  Every operation uses the explicitly rounded intrinsics so that the
// compiler can neither contract nor reorder them.
#pragma once

namespace ppgpu {

struct dfl {
    float h, l;
};

__device__ __forceinline__ dfl two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dfl two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    const dfl s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

// a + b without the final renormalisation (lo may exceed half an ulp of hi; the value is exact
// to the same order).  Used inside reductions that renormalise once at the end.
__device__ __forceinline__ dfl df_add_raw(dfl a, dfl b) {
    const dfl s = two_sum(a.h, b.h);
    return {s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l))};
}

__device__ __forceinline__ dfl df_add_f(dfl a, float b) {
    const dfl s = two_sum(a.h, b);
    return fast_two_sum(s.h, __fadd_rn(s.l, a.l));
}

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const dfl p = two_prod(a.h, b.h);
    const float e = __fmaf_rn(a.l, b.h, __fmaf_rn(a.h, b.l, p.l));
    return fast_two_sum(p.h, e);
}

__device__ __forceinline__ dfl df_mul_f(dfl a, float b) {
    const dfl p = two_prod(a.h, b);
    return fast_two_sum(p.h, __fmaf_rn(a.l, b, p.l));
}

__device__ __forceinline__ dfl df_sq(dfl a) {
    const dfl p = two_prod(a.h, a.h);
    return fast_two_sum(p.h, __fmaf_rn(__fadd_rn(a.h, a.h), a.l, p.l));
}

__host__ __device__ __forceinline__ dfl df_from(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

__device__ __forceinline__ double df_to(dfl a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ float df_round(dfl a) { return __fadd_rn(a.h, a.l); }

__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.h, -a.l}; }

// a / b: a quotient of the high parts, corrected once from the remainder a - q b (formed
// with TwoProduct), as in the double-word division of Dekker.
__device__ __forceinline__ dfl df_div(dfl a, dfl b) {
    const float q1 = __fdiv_rn(a.h, b.h);
    const dfl p = two_prod(q1, b.h);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.h, p.h), p.l), __fsub_rn(a.l, __fmul_rn(q1, b.l)));
    return fast_two_sum(q1, __fdiv_rn(r, b.h));
}

// a < b for normalised double-floats.
__device__ __forceinline__ bool df_lt(dfl a, dfl b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }

// floor(x) as a float and an int for |x| < 2^22 with float32 adds only (no conversion
// instructions): x + 1.5*2^23 rounds x to the nearest integer, held in the low mantissa bits.
__device__ __forceinline__ float floor_small(float x, int &i) {
    const float M = 12582912.0f;
    const float xm = __fadd_rn(x, M);
    float r = __fsub_rn(xm, M);
    int ri = __float_as_int(xm) - 0x4B400000;
    const bool over = r > x;
    r = over ? __fsub_rn(r, 1.f) : r;
    i = over ? ri - 1 : ri;
    return r;
}

// Integer + fraction of a double-float coordinate g: g = i + (t.h + t.l), t.h in [0, 1]
// exactly representable (the fraction bits of g.h), t.l = g.l.  |g| < 2^22.
__device__ __forceinline__ dfl split_cell(dfl g, int &i) {
    const float fl = floor_small(g.h, i);
    float th = __fsub_rn(g.h, fl);
    const bool below = (th == 0.f) && (g.l < 0.f);  // just under the boundary: previous cell
    th = below ? 1.f : th;
    i = below ? i - 1 : i;
    return {th, g.l};
}

}  // namespace ppgpu
