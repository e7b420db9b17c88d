// Host check of ffmath.cuh (the conditioning's Box-Muller pair in float-float with a
// rounding test) against the double evaluation the reference makes (Gaussian.cpp:23-35,
// divided by sqrt(2)_f and by the splat scale, rounded to float): every pair the test
// accepts must round to the double evaluation's floats.  Compiled by test_ffmath.py
// with -ffp-contract=off, so every float operation is one IEEE rounding as on the GPU.
#include "../gpis_extend_gb300/csrc/ffmath.cuh"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

static uint64_t g_state = 88172645463325252ull;
static uint32_t next_u32()
{
    g_state ^= g_state << 13;
    g_state ^= g_state >> 7;
    g_state ^= g_state << 17;
    return (uint32_t)(g_state >> 11);
}

// unit_float of a 32-bit draw: 23 random bits below 1
static float grid(uint32_t k) { return (float)(k & 0x7FFFFFu) * 0x1p-23f; }

static void reference(float u1, float u2, float sc, float &g0, float &g1)
{
    const double r = std::sqrt(-2.0 * std::log(1.0 - (double)u1));
    const float two_pi = 2.0f * 3.1415926536f;
    const double th = (double)two_pi * (double)u2;
    const double s2 = 1.4142135381698608;
    const double xs = 1.0 / (double)sc;
    g0 = (float)(r * std::cos(th) / s2 * xs);
    g1 = (float)(r * std::sin(th) / s2 * xs);
}

static long g_checked = 0, g_fallback = 0, g_bad = 0;

static void check(float u1, float u2, float sc)
{
    float a0, a1, b0, b1;
    ++g_checked;
    if (!ffm_normal_pair(u1, u2, sc, a0, a1)) {
        ++g_fallback;
        return;
    }
    reference(u1, u2, sc, b0, b1);
    if (ffm_bits(a0) != ffm_bits(b0) || ffm_bits(a1) != ffm_bits(b1)) {
        if (g_bad < 5) std::printf("mismatch u1=%a u2=%a sc=%a: %a %a against %a %a\n", u1, u2, sc, a0, a1, b0, b1);
        ++g_bad;
    }
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 4000000;
    for (long i = 0; i < n; ++i) {
        const float u1 = grid(next_u32()), u2 = grid(next_u32());
        const float sc = (i & 3) ? 1.0f : 0.25f + (float)(next_u32() & 0xFFFFFF) * 0x1p-24f * 1.5f;
        check(u1, u2, sc);
    }
    // every u1 against one angle, every angle against one u1
    for (uint32_t k = 0; k < (1u << 23); k += 3) {
        check(grid(k), grid(6421011u), 1.0f);
        check(grid(1035631u), grid(k), 1.0f);
    }
    std::printf("checked %ld, fallbacks %ld (%.2e), mismatches %ld\n", g_checked, g_fallback,
                (double)g_fallback / (double)g_checked, g_bad);
    return g_bad == 0 && g_fallback < g_checked / 1000 ? 0 : 1;
}
