// Host check of sph_fix40_add / sph_fix40_value against the C library's round-half-to-even of
// t * 2^40: every float t in [0, 16] alone, seeded sums of SPH_FIX_TERMS terms (the most the
// 32-bit sums take) against the sum of the rounded terms, and every 97th t on grids moved by 2^f.
// Exit status 0 when all agree.
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>

#include "sph_fixpoint.cuh"

static long long rint40(float t) { return (long long)std::nearbyint((double)t * 1099511627776.0); }

int main() {
    std::fesetround(FE_TONEAREST);
    unsigned long long checked = 0, bad = 0;
    float top = SPH_FIX_TMAX;
    unsigned end;
    std::memcpy(&end, &top, sizeof end);
    for (unsigned b = 0; b <= end; ++b) {
        float t;
        std::memcpy(&t, &b, sizeof t);
        unsigned H = 0, L = 0;
        sph_fix40_add(t, H, L);
        const long long got = sph_fix40_value(H, L), want = rint40(t);
        ++checked;
        if (got != want && bad++ < 10) std::printf("t=%a (bits %08x): %lld != %lld\n", (double)t, b, got, want);
    }
    // sums: terms spread over [0, 16] in log scale, and runs of the largest terms
    uint64_t s = 0x9E3779B97F4A7C15ull;
    for (int trial = 0; trial < 200000; ++trial) {
        unsigned H = 0, L = 0;
        long long want = 0;
        for (int k = 0; k < SPH_FIX_TERMS; ++k) {
            s ^= s << 13; s ^= s >> 7; s ^= s << 17;
            float t;
            if (trial % 4 == 0) {
                t = SPH_FIX_TMAX - (float)(s & 0xff) * 1.9073486328125e-06f;
            } else {
                const double u = (double)(s >> 11) * (1.0 / 9007199254740992.0);
                t = (float)(16.0 * std::exp2(-50.0 * u));
            }
            sph_fix40_add(t, H, L);
            want += rint40(t);
        }
        ++checked;
        if (sph_fix40_value(H, L) != want && bad++ < 10)
            std::printf("sum %d: %lld != %lld\n", trial, sph_fix40_value(H, L), want);
    }
    // the grid moved by 2^f (a run's own mass scale against the context's): t * 2^f with the
    // constants' exponents moved by f gives the counts of t
    for (int f : {-60, -23, -1, 1, 9, 60}) {
        const unsigned b1 = SPH_FIX_B1 + ((unsigned)f << 23), b2 = SPH_FIX_B2 + ((unsigned)f << 23);
        float c1, c2;
        std::memcpy(&c1, &b1, sizeof c1);
        std::memcpy(&c2, &b2, sizeof c2);
        for (unsigned b = 0; b <= end; b += 97) {
            float t;
            std::memcpy(&t, &b, sizeof t);
            const float tf = std::ldexp(t, f);
            unsigned H = 0, L = 0;
            sph_fix40_add(tf, H, L, c1, c2, b1, b2);
            ++checked;
            if (sph_fix40_value(H, L) != rint40(t) && bad++ < 10)
                std::printf("f=%d t=%a: %lld != %lld\n", f, (double)t, sph_fix40_value(H, L), rint40(t));
        }
    }
    std::printf("checked %llu, mismatches %llu\n", checked, bad);
    return bad ? 1 : 0;
}
