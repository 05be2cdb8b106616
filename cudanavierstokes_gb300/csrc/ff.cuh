// ff.cuh -- double-float ("FP32 pair") arithmetic: a value is the unevaluated sum h + l of
// two FP32 numbers with |l| <= ulp(h)/2, about 48 significant bits (relative precision
// ~2^-48 against FP64's 2^-53) in FP32's exponent range.
//
// The operations are the double-word algorithms of Joldes, Muller and Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word arithmetic" (ACM TOMS 44,
// 2017), built on Knuth's 2Sum, Dekker's Fast2Sum and the FMA-based exact product:
//   +  "SloppyDWPlusDW" (Alg. 5, 11 FP32 operations): error <= ~u^2 (|x| + |y|), u = 2^-24,
//      the norm-wise bound of an FP64 sum with u^2 in place of 2^-53;
//   *  "DWTimesDW" in the form without the x_l y_l term (Alg. 11, 8 operations): relative
//      error <= 6 u^2;
//   fma(a, b, c): the product's head and unnormalised tail (the first 5 operations of the
//      product) enter the sloppy sum with c directly, 16 operations instead of 8 + 11.
// Every step uses the _rn intrinsics, which the compiler neither contracts into FMAs nor
// reassociates: the error-free transforms rely on each rounding happening as written.
//
// On this GPU an FP64 operation issues to 2 lanes per SM per cycle and an FP32 one to 128,
// so a pair operation of 9-20 FP32 instructions still has several times the FP64 rate.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

namespace cns {

struct ff {
    float h, l;
    ff() = default;
    __host__ __device__ constexpr ff(float a, float b) : h(a), l(b) {}
    // from an integer constant (0, 1, 2 in generic code); a template, so that no double
    // reaches it through a conversion to int
    template <typename I, typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
    __host__ __device__ constexpr ff(I x) : h((float)x), l(0.0f) {}
    // nearest pair to a double (compile-time constants fold; at run time two conversions
    // and one FP64 subtraction)
    __host__ __device__ explicit constexpr ff(double x) : h((float)x), l((float)(x - (double)(float)x)) {}
};

__device__ __forceinline__ ff fast_two_sum(float a, float b) {   // |a| >= |b| or a = 0
    const float s = __fadd_rn(a, b);
    return ff(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff(s, e);
}

__device__ __forceinline__ ff operator+(ff x, ff y) {
    const ff s = two_sum(x.h, y.h);
    const float w = __fadd_rn(s.l, __fadd_rn(x.l, y.l));
    return fast_two_sum(s.h, w);
}

__device__ __forceinline__ ff operator-(ff x) { return ff(-x.h, -x.l); }
__device__ __forceinline__ ff operator-(ff x, ff y) { return x + ff(-y.h, -y.l); }

// head ch and unnormalised tail cl of x y: ch + cl = x y (1 + e), |e| <= 6 u^2
__device__ __forceinline__ void mul_parts(ff x, ff y, float& ch, float& cl) {
    ch = __fmul_rn(x.h, y.h);
    const float cl1 = __fmaf_rn(x.h, y.h, -ch);
    cl = __fadd_rn(cl1, __fmaf_rn(x.l, y.h, __fmul_rn(x.h, y.l)));
}

__device__ __forceinline__ ff operator*(ff x, ff y) {
    float ch, cl;
    mul_parts(x, y, ch, cl);
    return fast_two_sum(ch, cl);
}

// the pair overload joins the FP32 / FP64 ones (a namespace-scope fma would hide them)
using ::fma;
__device__ __forceinline__ ff fma(ff a, ff b, ff c) {
    float ph, pl;
    mul_parts(a, b, ph, pl);
    const ff s = two_sum(ph, c.h);
    const float w = __fadd_rn(s.l, __fadd_rn(pl, c.l));
    return fast_two_sum(s.h, w);
}

__device__ __forceinline__ ff& operator+=(ff& a, ff b) { a = a + b; return a; }
__device__ __forceinline__ ff& operator-=(ff& a, ff b) { a = a - b; return a; }
__device__ __forceinline__ ff& operator*=(ff& a, ff b) { a = a * b; return a; }

// Accumulator of a sum of products and pairs whose tail is not renormalised after each term
// (the compensated dot product of Ogita, Rump and Oishi, 2005, on pairs): the heads are
// summed exactly by 2Sum, the tail collects their rounding errors with the terms' tails, and
// one 2Sum normalises the result. 13 FP32 operations per product term (16 for fma) and 8 per
// added pair (11); the error stays at ~n u^2 times the largest term for n terms.
struct ffacc {
    float h, l;
    __device__ __forceinline__ explicit ffacc(ff x) : h(x.h), l(x.l) {}
    __device__ __forceinline__ void add_prod(ff a, ff b) {
        float ph, pl;
        mul_parts(a, b, ph, pl);
        const ff s = two_sum(h, ph);
        h = s.h;
        l = __fadd_rn(l, __fadd_rn(s.l, pl));
    }
    __device__ __forceinline__ void add(ff a) {
        const ff s = two_sum(h, a.h);
        h = s.h;
        l = __fadd_rn(l, __fadd_rn(s.l, a.l));
    }
    __device__ __forceinline__ ff value() const { return two_sum(h, l); }
};

// Two pairs side by side (lane x, lane y) through Blackwell's packed FP32x2 instructions
// (__fadd2_rn, __fmul2_rn, __ffma2_rn): the same algorithms as above, two independent pair
// operations per instruction sequence.
struct ff2 {
    float2 h, l;
};

__device__ __forceinline__ ff2 mk2(ff a, ff b) { return ff2{make_float2(a.h, b.h), make_float2(a.l, b.l)}; }
__device__ __forceinline__ ff lane0(ff2 v) { return ff(v.h.x, v.l.x); }
__device__ __forceinline__ ff lane1(ff2 v) { return ff(v.h.y, v.l.y); }

// negation and subtraction as one packed instruction each: b (-1) + a rounds once, exactly
// like a - b; a (-1) is exact
__device__ __forceinline__ float2 neg2(float2 a) { return __fmul2_rn(a, make_float2(-1.0f, -1.0f)); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

__device__ __forceinline__ void fast_two_sum2(float2 a, float2 b, float2& s, float2& e) {
    s = add2(a, b);
    e = sub2(b, sub2(s, a));
}
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
    s = add2(a, b);
    const float2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

__device__ __forceinline__ ff2 operator+(ff2 x, ff2 y) {
    float2 sh, sl, zh, zl;
    two_sum2(x.h, y.h, sh, sl);
    fast_two_sum2(sh, add2(sl, add2(x.l, y.l)), zh, zl);
    return ff2{zh, zl};
}
__device__ __forceinline__ ff2 operator-(ff2 x) { return ff2{neg2(x.h), neg2(x.l)}; }
__device__ __forceinline__ ff2 operator-(ff2 x, ff2 y) { return x + (-y); }

__device__ __forceinline__ void mul_parts2(ff2 x, ff2 y, float2& ch, float2& cl) {
    ch = __fmul2_rn(x.h, y.h);
    const float2 cl1 = __ffma2_rn(x.h, y.h, neg2(ch));
    cl = add2(cl1, __ffma2_rn(x.l, y.h, __fmul2_rn(x.h, y.l)));
}
__device__ __forceinline__ ff2 operator*(ff2 x, ff2 y) {
    float2 ch, cl, zh, zl;
    mul_parts2(x, y, ch, cl);
    fast_two_sum2(ch, cl, zh, zl);
    return ff2{zh, zl};
}
__device__ __forceinline__ ff2 fma(ff2 a, ff2 b, ff2 c) {
    float2 ph, pl, sh, sl, zh, zl;
    mul_parts2(a, b, ph, pl);
    two_sum2(ph, c.h, sh, sl);
    fast_two_sum2(sh, add2(sl, add2(pl, c.l)), zh, zl);
    return ff2{zh, zl};
}

// ffacc on two lanes
struct ffacc2 {
    float2 h, l;
    __device__ __forceinline__ explicit ffacc2(ff2 x) : h(x.h), l(x.l) {}
    __device__ __forceinline__ void add_prod(ff2 a, ff2 b) {
        float2 ph, pl, sh, sl;
        mul_parts2(a, b, ph, pl);
        two_sum2(h, ph, sh, sl);
        h = sh;
        l = add2(l, add2(sl, pl));
    }
    __device__ __forceinline__ void add(ff2 a) {
        float2 sh, sl;
        two_sum2(h, a.h, sh, sl);
        h = sh;
        l = add2(l, add2(sl, a.l));
    }
    __device__ __forceinline__ ff2 value() const {
        float2 zh, zl;
        two_sum2(h, l, zh, zl);
        return ff2{zh, zl};
    }
};

template <typename R>
inline constexpr bool is_ff = false;
template <>
inline constexpr bool is_ff<ff> = true;

// FP64 <-> pair: (double)h + (double)l rounds once in FP64 (2^-53, below the pair's own
// precision); the split rounds h, then the remainder x - h (exact in FP64)
__device__ __forceinline__ double ff_to_d(ff x) { return (double)x.h + (double)x.l; }
__device__ __forceinline__ ff d_to_ff(double x) {
    const float h = __double2float_rn(x);
    return ff(h, __double2float_rn(x - (double)h));
}

}  // namespace cns

// read-only cached load of a pair (one 8-byte load)
__device__ __forceinline__ cns::ff __ldg(const cns::ff* p) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return cns::ff(v.x, v.y);
}
