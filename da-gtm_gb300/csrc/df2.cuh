// df2.cuh -- two double-float computations at once on packed FP32 pairs
// (add / sub / mul / fma.rn.f32x2, sm_100+): the operations of df.cuh in the
// same order, lane by lane, so each lane's result is bitwise the scalar one.
// Lane 0 is the low half of each 64-bit register, lane 1 the high half.
// Used where two exponentials are independent: the two temperatures of one
// centre-point pair (pass 1) or two centres of one point (pass 2).
#pragma once

#include "df.cuh"
#include "sm100.cuh"

namespace dgtm {
namespace df2 {

using sm100::f2;
using sm100::f2_add;
using sm100::f2_hi;
using sm100::f2_lo;
using sm100::f2_mul;
using sm100::f2_pack;
using sm100::f2_sub;

__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}

__device__ __forceinline__ f2 neg2(f2 a)
{
    a.v ^= 0x8000000080000000ull;
    return a;
}

__device__ __forceinline__ f2 splat(float x) { return f2_pack(x, x); }

// two double-floats: (h.lane0, l.lane0) and (h.lane1, l.lane1)
struct x2 {
    f2 h, l;
};

__device__ __forceinline__ df::f2x lane0(x2 a) { return {f2_lo(a.h), f2_lo(a.l)}; }
__device__ __forceinline__ df::f2x lane1(x2 a) { return {f2_hi(a.h), f2_hi(a.l)}; }
__device__ __forceinline__ x2 pack(df::f2x a, df::f2x b) { return {f2_pack(a.h, b.h), f2_pack(a.l, b.l)}; }

__device__ __forceinline__ void two_sum(f2 a, f2 b, f2 &s, f2 &e)
{
    s = f2_add(a, b);
    const f2 bb = f2_sub(s, a);
    e = f2_add(f2_sub(a, f2_sub(s, bb)), f2_sub(b, bb));
}

__device__ __forceinline__ void fast_two_sum(f2 a, f2 b, f2 &s, f2 &e)
{
    s = f2_add(a, b);
    e = f2_sub(b, f2_sub(s, a));
}

__device__ __forceinline__ void two_prod(f2 a, f2 b, f2 &p, f2 &e)
{
    p = f2_mul(a, b);
    e = fma2(a, b, neg2(p));
}

// df::add lane by lane
__device__ __forceinline__ x2 add(x2 a, x2 b)
{
    f2 s1, s2, t1, t2;
    two_sum(a.h, b.h, s1, s2);
    two_sum(a.l, b.l, t1, t2);
    s2 = f2_add(s2, t1);
    fast_two_sum(s1, s2, s1, s2);
    s2 = f2_add(s2, t2);
    fast_two_sum(s1, s2, s1, s2);
    return {s1, s2};
}

// df::sum4 lane by lane
__device__ __forceinline__ x2 sum4(f2 u, f2 v, f2 w1, f2 w2)
{
    x2 a, b;
    two_sum(u, v, a.h, a.l);
    two_sum(w1, w2, b.h, b.l);
    return add(a, b);
}

// df::mul lane by lane
__device__ __forceinline__ x2 mul(x2 a, x2 b)
{
    f2 p, e;
    two_prod(a.h, b.h, p, e);
    e = fma2(a.h, b.l, e);
    e = fma2(a.l, b.h, e);
    fast_two_sum(p, e, p, e);
    return {p, e};
}

// df::exp_df lane by lane (0 below df::EXP_CUT in each lane)
template <typename TAB>
__device__ __forceinline__ x2 exp_df(x2 x, const TAB &tab)
{
    using namespace df;
    const float xh0 = f2_lo(x.h), xh1 = f2_hi(x.h);
    const f2 km = f2_mul(x.h, splat(EXP_INV));
    const float kf0 = rintf(f2_lo(km)), kf1 = rintf(f2_hi(km));
    const f2 kf = f2_pack(kf0, kf1);
    const int k0 = (int) kf0, k1 = (int) kf1;
    const f2 r1 = fma2(neg2(kf), splat(EXP_L1), x.h);
    f2 p2, e2;
    two_prod(kf, splat(EXP_L2), p2, e2);
    f2 s, t, s2, t2;
    two_sum(r1, neg2(p2), s, t);
    two_sum(s, x.l, s2, t2);
    const f2 lo = f2_add(f2_add(t, t2), neg2(fma2(kf, splat(EXP_L3), e2)));
    f2 rh, rl;
    fast_two_sum(s2, lo, rh, rl);
    f2 r2h, r2l;
    two_prod(rh, rh, r2h, r2l);
    r2l = fma2(f2_mul(splat(2.0f), rh), rl, r2l);
    f2 t3, e3;
    two_prod(rh, r2h, t3, e3);
    e3 = fma2(rh, r2l, e3);
    const f2 r4 = f2_mul(t3, rh);
    const f2 c = fma2(r4, fma2(rh, splat(1.0f / 120.0f), splat(1.0f / 24.0f)),
                      fma2(t3, splat(SIXTH_H), fma2(e3, splat(SIXTH_H), f2_mul(t3, splat(SIXTH_L)))));
    f2 ph, pl;
    two_sum(rh, f2_mul(splat(0.5f), r2h), ph, pl);
    pl = f2_add(pl, f2_add(f2_add(rl, f2_mul(splat(0.5f), r2l)), c));
    fast_two_sum(ph, pl, ph, pl);
    const int j0 = k0 & 63, j1 = k1 & 63;
    const f2 Th = f2_pack(tab[j0].x, tab[j1].x), Tl = f2_pack(tab[j0].y, tab[j1].y);
    f2 mh, me;
    two_prod(Th, ph, mh, me);
    me = fma2(Th, pl, me);
    me = fma2(Tl, ph, me);
    f2 eh, el;
    two_sum(Th, mh, eh, el);
    el = f2_add(el, f2_add(Tl, me));
    fast_two_sum(eh, el, eh, el);
    // 2^m per lane; a lane below the cut (or NaN) is 0 whatever the rest made of it
    const f2 sc = f2_pack(__uint_as_float((uint32_t) ((k0 >> 6) + 127) << 23),
                          __uint_as_float((uint32_t) ((k1 >> 6) + 127) << 23));
    const uint64_t keep = ((xh0 >= EXP_CUT) ? 0x00000000FFFFFFFFull : 0ull) |
                          ((xh1 >= EXP_CUT) ? 0xFFFFFFFF00000000ull : 0ull);
    x2 r = {f2_mul(eh, sc), f2_mul(el, sc)};
    r.h.v &= keep;
    r.l.v &= keep;
    return r;
}

}  // namespace df2
}  // namespace dgtm
