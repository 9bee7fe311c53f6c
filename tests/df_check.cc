// Host check of the double-float arithmetic of the exact-slice FP64 form
// (da-gtm_gb300/csrc/df.cuh) against long-double and exact integer results.
// Prints one line per function: the largest error seen and the bound.
// Built with -ffp-contract=off (the error-free transformations need every
// operation rounded on its own).
#include "../da-gtm_gb300/csrc/df.cuh"

#include <math.h>
#include <stdint.h>
#include <stdio.h>

using namespace dgtm::df;

namespace {

struct ent {
    float x, y;
};

uint64_t rng_state = 0x9E3779B97F4A7C15ull;

uint64_t next_u64()
{
    // splitmix64
    uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform() { return (double) (next_u64() >> 11) * (1.0 / 9007199254740992.0); }

long double ld(f2x a) { return (long double) a.h + (long double) a.l; }

}  // namespace

int main()
{
    ent tab[64];
    for (int j = 0; j < 64; j++)
        exp_table_entry(j, tab[j].x, tab[j].y);
    const int n = 2000000;

    // exp on [-45, 1] (double-float arguments with a full low part)
    long double emax = 0.0L;
    double worst_x = 0.0;
    for (int i = 0; i < n; i++) {
        double xd;
        if (i % 4 == 0)
            xd = -45.0 * uniform();
        else if (i % 4 == 1)
            xd = -0.05 * uniform();  // near 0, where R is large
        else if (i % 4 == 2)
            xd = 1.0 - 2.0 * uniform();
        else
            xd = -(double) (next_u64() % 2880) / 64.0 + 1e-9 * (uniform() - 0.5);  // table edges
        const f2x x = from_double(xd);
        const f2x e = exp_df(x, tab);
        const long double ref = expl(ld(x));
        const long double rel = fabsl(ld(e) - ref) / ref;
        if (rel > emax) {
            emax = rel;
            worst_x = xd;
        }
    }
    printf("exp_df max_rel %.3Le at x=%.17g\n", emax, worst_x);
    // below the cut: 0
    const f2x z = exp_df(from_double(-45.5), tab);
    printf("exp_df below_cut %g %g\n", z.h, z.l);

    // sum4: the recombination of exact slice partials u = d0 2^40, v = d1 2^24,
    // w1 = d2 2^8, w2 = d3 with |d| < 2^24, often nearly cancelling
    long double smax = 0.0L;
    for (int i = 0; i < n; i++) {
        int32_t d[4];
        for (int q = 0; q < 4; q++)
            d[q] = (int32_t) (next_u64() % (1u << 25)) - (1 << 24) + 1;
        if (i % 3 == 0) {
            d[0] = (int32_t) (next_u64() % 5) - 2;  // small differences, cancellation
            d[1] = (int32_t) (next_u64() % 512) - 256;
        }
        __int128 exact = ((__int128) d[0] << 40) + ((__int128) d[1] << 24) + ((__int128) d[2] << 8) +
                         (__int128) d[3];
        const f2x s = sum4(ldexpf((float) d[0], 40), ldexpf((float) d[1], 24), ldexpf((float) d[2], 8),
                           (float) d[3]);
        if (exact == 0) {
            if (s.h != 0.f || s.l != 0.f)
                smax = 1.0L;
            continue;
        }
        const long double ex = (long double) exact;
        const long double rel = fabsl(ld(s) - ex) / fabsl(ex);
        if (rel > smax)
            smax = rel;
    }
    printf("sum4 max_rel %.3Le\n", smax);

    // mul
    long double mmax = 0.0L;
    for (int i = 0; i < n; i++) {
        const f2x a = from_double((uniform() - 0.5) * 1e3), b = from_double((uniform() - 0.5) * 1e-3);
        const f2x p = mul(a, b);
        const long double ref = ld(a) * ld(b);
        const long double rel = fabsl(ld(p) - ref) / fabsl(ref);
        if (rel > mmax)
            mmax = rel;
    }
    printf("mul max_rel %.3Le\n", mmax);

    // fixed48: round(E 2^48) for E in [0, 2), within one unit
    long double fmax = 0.0L;
    for (int i = 0; i < n; i++) {
        double ed = (i % 3 == 0) ? uniform() * 2.0 : (i % 3 == 1) ? uniform() * 1e-6 : 1.0 - uniform() * 1e-9;
        f2x e = from_double(ed);
        if (i % 7 == 0) {  // integer top with a negative low part
            // and tops at and above 1, where E 2^24 is an even integer
            const float h = (i % 2) ? ldexpf(rintf(ldexpf((float) uniform(), 24)), -24)
                                    : 1.0f + ldexpf(rintf(ldexpf((float) uniform(), 23)), -23);
            int ex;
            frexpf(h, &ex);
            e = {h, -(float) uniform() * ldexpf(1.0f, ex - 25)};  // |l| <= ulp(h) / 2
            if (h == 0.f)
                e.l = 0.f;
        }
        const uint64_t f = fixed48(e);
        const long double ref = ldexpl(ld(e), 48);
        const long double err = fabsl((long double) f - ref);
        if (err > fmax)
            fmax = err;
    }
    printf("fixed48 max_abs_units %.3Lf\n", fmax);

    // fixed48r: the integers plus the FP32 sum of remainders against the
    // long-double sum of 60000 terms below 1 (the largest K), several times
    long double rmax = 0.0L;
    for (int rep = 0; rep < 20; rep++) {
        uint64_t si = 0;
        float sr = 0.f;
        long double ls = 0.0L;
        for (int i = 0; i < 60000; i++) {
            const double ed = (i % 2) ? uniform() : ldexp(uniform(), -(int) (next_u64() % 45));
            const f2x e = from_double(ed);
            float r;
            si += fixed48r(e, r);
            sr += r;
            ls += ld(e);
        }
        const long double got = ldexpl((long double) si + (long double) sr, -48);
        const long double relr = fabsl(got - ls) / ls;
        if (relr > rmax)
            rmax = relr;
    }
    printf("fixed48r sum_rel %.3Le\n", rmax);
    return 0;
}
