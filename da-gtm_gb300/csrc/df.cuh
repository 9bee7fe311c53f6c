// df.cuh -- double-float arithmetic (a value held as an unevaluated sum of two
// FP32 numbers, ~48 significant bits) for the exact-slice FP64 form.
//
// GB300 issues FP64 at about 1/64 of its FP32 rate, so the form that keeps
// FP64 accuracy does its O(K N) arithmetic on the FP32 pipe: the distance
// products are exact integers from the tensor cores (estep_x64.cu), and the
// exponentials and fixed-point conversions below work on FP32 pairs.  Only
// O(N + K) work (logarithms, per-point and per-centre terms) stays in FP64.
//
// Everything here is host/device code so that the same functions can be
// checked on the CPU against long-double references.  The error-free
// transformations use explicitly rounded operations (no contraction into FMA
// behind their back); the host build needs -ffp-contract=off.
//
// Methods: TwoSum (Knuth), FastTwoSum (Dekker), TwoProduct via FMA; the
// accurate double-word addition of Li et al. (the "IEEE" variant of the QD
// library's dd_add); exp by Tang's table method: x = k ln2/64 + r with
// |r| <= ln2/128, exp(x) = 2^(k div 64) 2^((k mod 64)/64) exp(r), exp(r) by
// its Taylor series to degree 5 (truncation below 2^-54).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD static inline
#endif

namespace dgtm {
namespace df {

struct f2x {
    float h, l;
};

DF_HD float add_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

DF_HD float sub_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

DF_HD float mul_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

// s + e == a + b exactly, s = fl(a + b)
DF_HD void two_sum(float a, float b, float &s, float &e)
{
    s = add_rn(a, b);
    const float bb = sub_rn(s, a);
    e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
}

// the same for |a| >= |b| (or a == 0)
DF_HD void fast_two_sum(float a, float b, float &s, float &e)
{
    s = add_rn(a, b);
    e = sub_rn(b, sub_rn(s, a));
}

// p + e == a b exactly
DF_HD void two_prod(float a, float b, float &p, float &e)
{
    p = mul_rn(a, b);
    e = fmaf(a, b, -p);
}

// a + b with relative error below 3 2^-48, cancellation included
DF_HD f2x add(f2x a, f2x b)
{
    float s1, s2, t1, t2;
    two_sum(a.h, b.h, s1, s2);
    two_sum(a.l, b.l, t1, t2);
    s2 = add_rn(s2, t1);
    fast_two_sum(s1, s2, s1, s2);
    s2 = add_rn(s2, t2);
    fast_two_sum(s1, s2, s1, s2);
    return {s1, s2};
}

// a b (relative error below 4 2^-48)
DF_HD f2x mul(f2x a, f2x b)
{
    float p, e;
    two_prod(a.h, b.h, p, e);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    fast_two_sum(p, e, p, e);
    return {p, e};
}

// The double-float nearest (to 48 bits) of u + v + w1 + w2, four exact FP32
// values: the recombination of the slice partials of an exact integer.
DF_HD f2x sum4(float u, float v, float w1, float w2)
{
    f2x a, b;
    two_sum(u, v, a.h, a.l);
    two_sum(w1, w2, b.h, b.l);
    return add(a, b);
}

// FP64 value -> double-float (48 of its 53 bits)
DF_HD f2x from_double(double x)
{
    const float h = (float) x;
    return {h, (float) (x - (double) h)};
}

DF_HD double to_double(f2x a) { return (double) a.h + (double) a.l; }

// ---------------------------------------------------------------- exp
// ln2/64 = L1 + L2 + L3: L1 has 9 significant bits (k L1 is exact for
// |k| < 2^15), L2 and L3 the next two FP32 pieces.
constexpr double LN2_64 = 0.69314718055994530942 / 64.0;
constexpr float EXP_L1 = 355.0f / 32768.0f;
constexpr float EXP_L2 = (float) (LN2_64 - (double) EXP_L1);
constexpr float EXP_L3 = (float) ((LN2_64 - (double) EXP_L1) - (double) EXP_L2);
constexpr float EXP_INV = (float) (64.0 / 0.69314718055994530942);
// 1/6 as a double-float
constexpr float SIXTH_H = (float) (1.0 / 6.0);
constexpr float SIXTH_L = (float) (1.0 / 6.0 - (double) SIXTH_H);
// below this argument exp(x) < 2^-64: the per-point sums and the
// responsibilities (2^-48 fixed point) take it as 0; K such terms change a
// sum of at least 1 by less than 2^-48 for K < 2^16
constexpr float EXP_CUT = -45.0f;

// The table 2^(j/64), j = 0..63, as double-floats (tab[j] = {hi, lo}).
DF_HD void exp_table_entry(int j, float &h, float &l)
{
    const double v = exp2((double) j / 64.0);
    h = (float) v;
    l = (float) (v - (double) h);
}

// exp(x) for x <= 1 with relative error about 2^-47; 0 below EXP_CUT.
// tab: the 64-entry table (shared memory on the device).
template <typename TAB>
DF_HD f2x exp_df(f2x x, const TAB &tab)
{
    if (!(x.h >= EXP_CUT))
        return {0.f, 0.f};
    const float kf = rintf(mul_rn(x.h, EXP_INV));
    const int k = (int) kf;
    // r = x - k ln2/64 (exact r1; k L2 split exactly; k L3 rounded far below 2^-52)
    const float r1 = fmaf(-kf, EXP_L1, x.h);
    float p2, e2;
    two_prod(kf, EXP_L2, p2, e2);
    // r1 - p2 + x.l exactly as s2 + t + t2 (x.l reaches 2^-20 at |x| = 36),
    // then the terms below 2^-30, whose roundings stay below 2^-54
    float s, t, s2, t2;
    two_sum(r1, -p2, s, t);
    two_sum(s, x.l, s2, t2);
    const float lo = add_rn(add_rn(t, t2), -fmaf(kf, EXP_L3, e2));
    float rh, rl;
    fast_two_sum(s2, lo, rh, rl);
    // exp(r) - 1 = r + r^2/2 + r^3/6 + r^4 (1/24 + r/120)
    float r2h, r2l;
    two_prod(rh, rh, r2h, r2l);
    r2l = fmaf(mul_rn(2.0f, rh), rl, r2l);
    float t3, e3;
    two_prod(rh, r2h, t3, e3);  // r^3 = t3 + e3 (+ rh r2l)
    e3 = fmaf(rh, r2l, e3);
    const float r4 = mul_rn(t3, rh);
    const float c = fmaf(r4, fmaf(rh, 1.0f / 120.0f, 1.0f / 24.0f),
                         fmaf(t3, SIXTH_H, fmaf(e3, SIXTH_H, mul_rn(t3, SIXTH_L))));
    float ph, pl;
    two_sum(rh, mul_rn(0.5f, r2h), ph, pl);
    pl = add_rn(pl, add_rn(add_rn(rl, mul_rn(0.5f, r2l)), c));
    fast_two_sum(ph, pl, ph, pl);
    // 2^(j/64) (1 + p)
    const int j = k & 63, m = k >> 6;
    const float Th = tab[j].x, Tl = tab[j].y;
    float mh, me;
    two_prod(Th, ph, mh, me);
    me = fmaf(Th, pl, me);
    me = fmaf(Tl, ph, me);
    float eh, el;
    two_sum(Th, mh, eh, el);
    el = add_rn(el, add_rn(Tl, me));
    fast_two_sum(eh, el, eh, el);
    // 2^m, m in [-65, 2]
    union {
        uint32_t u;
        float f;
    } sc;
    sc.u = (uint32_t) (m + 127) << 23;
    return {mul_rn(eh, sc.f), mul_rn(el, sc.f)};
}

// ---------------------------------------------------------------- fixed point
// round(E 2^48) for 0 <= E < 2 (E a normalised double-float), as a 24-bit top
// and a bottom in [0, 2^24] whose sum top 2^24 + bottom is the result.
DF_HD void fixed48_parts(f2x e, uint32_t &top, uint32_t &bot)
{
    const float z = mul_rn(e.h, 16777216.0f);  // exact
    const float zf = floorf(z);
    const float lz = mul_rn(e.l, 16777216.0f);  // |lz| <= ulp(z) / 2
    // z an integer and the low part negative: the top is z - 1 (in integers:
    // above 2^24, z - 1 is not an FP32 number)
    const bool dec = (zf == z) && (lz < 0.f);
    top = (uint32_t) zf - (dec ? 1u : 0u);
    // in [0, 1]: the fraction of E 2^24 above the top
    const float frac = dec ? add_rn(1.0f, lz) : add_rn(sub_rn(z, zf), lz);
    bot = (uint32_t) rintf(mul_rn(frac, 16777216.0f));
}

DF_HD uint64_t fixed48(f2x e)
{
    uint32_t top, bot;
    fixed48_parts(e, top, bot);
    return ((uint64_t) top << 24) + (uint64_t) bot;
}

// round(E 2^48) for 0 <= E < 2 as fixed48, and the rounding remainder
// E 2^48 - round(E 2^48) in [-1/2, 1/2] to ~2^-24 of itself: a sum of many
// terms is exact to 2^-48 in the integers plus the FP32 sum of remainders.
DF_HD uint64_t fixed48r(f2x e, float &rem)
{
    const float z = mul_rn(e.h, 16777216.0f);  // exact
    const float zf = floorf(z);
    const float lz = mul_rn(e.l, 16777216.0f);
    const bool dec = (zf == z) && (lz < 0.f);
    const uint32_t top = (uint32_t) zf - (dec ? 1u : 0u);
    // the fraction above the top, exactly: fs + fe
    float fs, fe;
    two_sum(dec ? 1.0f : sub_rn(z, zf), lz, fs, fe);
    const float scaled = mul_rn(fs, 16777216.0f);  // exact
    const float bf = rintf(scaled);
    rem = fmaf(fe, 16777216.0f, sub_rn(scaled, bf));
    return ((uint64_t) top << 24) + (uint64_t) (uint32_t) bf;
}

}  // namespace df
}  // namespace dgtm
